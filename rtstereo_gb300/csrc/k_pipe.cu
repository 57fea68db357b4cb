// k_pipe.cu -- fused per-view pipeline kernels.
//
// Every fused kernel keeps the reference's per-entry arithmetic (the same
// operands combined in the same order with round-to-nearest float ops), so the
// fused pipeline is bit-identical to the composed module kernels and to the
// reference; fusion only removes HBM round trips and adds on-chip reuse.
//
//   k_prep_records  per pixel one 16-byte record: 64-bit census code, packed
//                   RGB, packed cross arms (l | r<<8 | t<<16 | b<<24)
//   k_cost_volume   AD / census / AD+census(CombineCost) cost volume from records
//   (the cross-based stages work over view tables and live in k_batch.cu)
//   k_aw_wta        adaptive-weight aggregation (seq/AdaptiveWeightAggregation.cpp:73-111)
//                   over 64-pixel x 64-disparity tiles, weights made on the fly from
//                   Lab + host tables, and the arg-min over d
#include <algorithm>

#include "rts_fused.cuh"
#include "rts_pipe.h"
#include "rts_tma.h"

namespace rts {

// ---------------------------------------------------------------------------
__global__ void k_prep_records(const uint8_t *__restrict__ gray, const uint8_t *__restrict__ rgb,
                               uint4 *__restrict__ rec, uint32_t *__restrict__ arms_out, int H, int W, int hr, int wr,
                               int L, int tau, int want_code, int want_arms) {
    const int y = blockIdx.y;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    const long p = (long)y * W + x;
    uint64_t code = 0;
    if (want_code) {
        // seq/CensusTransform.cpp:11-37, bit (dy+hr)*(2wr+1)+(dx+wr), strict centre > neighbour
        const uint8_t c = gray[p];
        int k = 0;
        if (x >= wr && x < W - wr && y >= hr && y < H - hr) {
            // the window inside the image: no wrapping
            const uint8_t *row = gray + p - (size_t)hr * W - wr;
            for (int dy = -hr; dy <= hr; dy++, row += W)
                for (int dx = 0; dx <= 2 * wr; dx++, k++) code |= (uint64_t)(c > row[dx]) << k;
        } else {
            for (int dy = -hr; dy <= hr; dy++) {
                const uint8_t *row = gray + (size_t)wrap1(y + dy, H) * W;
                for (int dx = -wr; dx <= wr; dx++, k++) code |= (uint64_t)(c > row[wrap1(x + dx, W)]) << k;
            }
        }
    }
    const uint8_t *px = rgb + 3 * p;
    const uint32_t packed = (uint32_t)px[0] | ((uint32_t)px[1] << 8) | ((uint32_t)px[2] << 16);
    uint32_t arms = 0;
    if (want_arms) {
        // seq/CrossBasedAggregation.cpp:12-100, same stepping rule as k_find_cross
        const int c0 = px[0], c1 = px[1], c2 = px[2];
        int len[4];
        const long step[4] = {-1, 1, -(long)W, (long)W};
        const int room[4] = {x, W - 1 - x, y, H - 1 - y};
#pragma unroll
        for (int a = 0; a < 4; a++) {
            int n = 0, delta = 0;
            while (delta < tau && n < L && n < room[a]) {
                n++;
                const uint8_t *q = rgb + 3 * (p + step[a] * n);
                delta = imax(imax(abs(c0 - (int)q[0]), abs(c1 - (int)q[1])), abs(c2 - (int)q[2]));
            }
            len[a] = n;
        }
        arms = (uint32_t)len[0] | ((uint32_t)len[1] << 8) | ((uint32_t)len[2] << 16) | ((uint32_t)len[3] << 24);
    }
    rec[p] = make_uint4((uint32_t)code, (uint32_t)(code >> 32), packed, arms);
    if (arms_out) arms_out[p] = arms;
}

// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_cost_volume(const uint4 *__restrict__ rr, const uint4 *__restrict__ rt, T *__restrict__ vol, int H,
                              int W, int D, CostCfg cfg) {
    const int y = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * D) return;
    const int x = i / D, d = i - x * D;
    const int xt = tar_col(x, d, W, 1);
    const uint4 a = rr[(size_t)y * W + x], b = rt[(size_t)y * W + xt];
    vol[((size_t)y * W + x) * D + d] = to_store<T>(pair_cost(a, b, cfg));
}

// AD (optionally truncated) + census combined through the two host tables, the
// integer path: warp per pixel, lane = disparity, so the reference record is a
// broadcast and the volume row is contiguous.  Block per (row, 64 pixels): the
// target records the block meets, columns x0 - D + 1 .. x0 + 63 (wrapped as in
// seq/PixelBasedCost.cpp:19-20), and the two tables are staged in shared memory
// once, so an entry reads its target record (consecutive lanes, consecutive
// records) and its two table values from shared memory.
constexpr int kAdcPx = 8;
constexpr int kAdcTX = 8 * kAdcPx;          // pixels of a block
constexpr int kAdcL1 = 768, kAdcL2 = 68;    // table entries staged: AD <= 765, census <= 64
template <typename T>
__global__ void __launch_bounds__(256) k_cost_volume_adc(const uint4 *__restrict__ rr, const uint4 *__restrict__ rt,
                                                        T *__restrict__ vol, int H, int W, int D, int itrunc,
                                                        const float *__restrict__ lut1, const float *__restrict__ lut2) {
    __shared__ uint4 trec[kAdcTX + 255];  // D <= 256
    __shared__ float t1[kAdcL1], t2[kAdcL2];
    const int y = blockIdx.y, lane = threadIdx.x & 31, tid = threadIdx.x;
    const int x0 = blockIdx.x * kAdcTX, base = x0 - D + 1;
    const uint4 *trow = rt + (size_t)y * W;
    for (int i = tid; i < kAdcTX + D - 1; i += 256) {
        int xt = base + i;
        if (xt < 0) xt += W;  // seq/PixelBasedCost.cpp:19-20 (D <= W)
        trec[i] = trow[imin(xt, W - 1)];  // columns past the row end are never read
    }
    for (int i = tid; i < kAdcL1; i += 256) t1[i] = lut1[i];
    if (tid < kAdcL2) t2[tid] = lut2[tid];
    __syncthreads();
    // a warp takes kAdcPx consecutive pixels of the row
    const int xw = x0 + (tid >> 5) * kAdcPx;
#pragma unroll 2
    for (int i = 0; i < kAdcPx; i++) {
        const int x = xw + i;
        if (x >= W) return;
        const uint4 a = rr[(size_t)y * W + x];
        T *out = vol + ((size_t)y * W + x) * D;
        const uint4 *tb = trec + (x - base);  // target of disparity d: tb[-d]
        for (int d = lane; d < D; d += 32) {
            const uint4 b = tb[-d];
            const int sad = imin((int)__vsadu4(a.z, b.z), itrunc);    // seq/PixelBasedCost.cpp:86-91 / :106-112
            const int ham = __popc(a.x ^ b.x) + __popc(a.y ^ b.y);   // seq/CensusTransform.cpp:52-60
            out[d] = to_store<T>(__fadd_rn(t1[sad], t2[ham]));       // seq/CombineCost.cpp:23
        }
    }
}

// ---------------------------------------------------------------------------
// Adaptive-weight aggregation fused with the arg-min.  Block: one row y, 64
// pixels x0..x0+63, all disparities in chunks of 64; 256 threads, each with
// 4 pixels x 4 disparities.  Warp w owns pixels 8w..8w+7 for all 64
// disparities (lane = 2 pixel groups x 16 disparity groups), so the reference
// weights are broadcast loads and the target weights and costs are contiguous.
// Per tap row ky the block stages the cost rows (wrapped columns x0-r ..
// x0+63+r), the packed Lab rows of the tap row, then the reference weights
// wR(p, ky, kx) and the target weights wT(t, ky, kx) for t = x0-dc0-63 ..
// x0-dc0+63 (wrapped), then every thread adds its 32 chains in the reference's
// order (plain form):
//   w = wR*wT;  sw = sw + w;  sc = sc + C*w      (seq/AdaptiveWeightAggregation.cpp:100-103)
// Tap rows outside the image have all-zero weights and add exact zeros, so
// they are skipped.  A weight is pw[k] * G[|Lab(p)-Lab(q)|^2] with host tables
// (seq/AdaptiveWeightAggregation.cpp:60-63); |Lab(p)-Lab(q)|^2 is the dot
// product of the byte-wise absolute differences of the packed Lab words.
constexpr int kAwTX = 64, kAwDC = 64, kAwThreads = 256;
constexpr int kAwCPitch = kAwDC + 4;
constexpr int kAwHPitch = kAwDC + 8;  // f16 cost rows: 144 bytes, a multiple of 16
constexpr uint32_t kLabOut = 0xff000000u;  // marks a column outside the image

__global__ void k_pack_lab(const uint8_t *__restrict__ lab, uint32_t *__restrict__ out, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = (uint32_t)lab[3 * i] | ((uint32_t)lab[3 * i + 1] << 8) | ((uint32_t)lab[3 * i + 2] << 16);
}

template <typename CT, bool EXACT>
__global__ void __launch_bounds__(kAwThreads, 3) k_aw_wta(const CT *__restrict__ vol, const uint32_t *__restrict__ labr,
                                                      const uint32_t *__restrict__ labt, const float *__restrict__ pw,
                                                      const float *__restrict__ G, uint16_t *__restrict__ raw,
                                                      int *__restrict__ row_last, float *__restrict__ cost_out, int H,
                                                      int W, int D, int e) {
    // EXACT: the reference's unfused w*C then add (plain form); otherwise one fma
    const int r = e >> 1;
    constexpr int NT = kAwTX + kAwDC - 1;  // target columns of a tile
    constexpr int NTP = NT + 1;
    extern __shared__ __align__(16) float asm_[];
    float *Cs = asm_;                                   // [(64+2r+4)][kAwCPitch], 4 spare rows
    float *wRs = Cs + (kAwTX + 2 * r + 4) * kAwCPitch;  // [e][64]
    float *wTs = wRs + e * kAwTX;                       // [e][NTP]
    uint32_t *labRrow = reinterpret_cast<uint32_t *>(wTs + e * NTP);  // [64 + 2r]
    uint32_t *labTrow = labRrow + (kAwTX + 2 * r);                    // [NT + 2r]
    __shared__ float best_v[kAwTX];
    __shared__ int best_i[kAwTX];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int td = lane & 15;                      // disparities 4td .. 4td+3 of the chunk
    const int px0 = 8 * warp + 4 * (lane >> 4);  // pixels px0 .. px0+3 of the tile
    const int y = blockIdx.y, x0 = blockIdx.x * kAwTX;
    if (tid < kAwTX) {
        best_v[tid] = __int_as_float(0x7f800000);
        best_i[tid] = 0x7fffffff;
    }
    const bool vec = (D & 3) == 0;

    for (int dc0 = 0; dc0 < D; dc0 += kAwDC) {
        // sums of disparity pairs (4td + 2h, 4td + 2h + 1) of pixel px0 + j, packed for
        // the f32x2 instructions (each half an IEEE round-to-nearest operation)
        unsigned long long sw[4][2], sc[4][2];
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int h = 0; h < 2; h++) sw[j][h] = sc[j][h] = 0ull;
        // centre Lab words: reference pixels x0+lane+32m, target columns t(u), u = lane+32m
        const int tbase = x0 - dc0 - (kAwDC - 1);  // target column of u = 0, before wrapping
        uint32_t cR[2], cT[4];
#pragma unroll
        for (int m = 0; m < 2; m++) {
            const int x = x0 + lane + 32 * m;
            cR[m] = x < W ? labr[(size_t)y * W + x] : kLabOut;
        }
#pragma unroll
        for (int m = 0; m < 4; m++) {
            int t = tbase + lane + 32 * m;
            if (t < 0) t += W;  // seq/AdaptiveWeightAggregation.cpp:87
            cT[m] = (lane + 32 * m < NT && t >= 0 && t < W) ? labt[(size_t)y * W + t] : kLabOut;
        }
        // targets that wrapped around the left edge take their tap row from the
        // other end of the row; only tiles with tbase < 0 have them
        const bool wrapped_tile = tbase < 0;

        const int ky_lo = imax(-r, -y), ky_hi = imin(r, H - 1 - y);
        for (int ky = ky_lo; ky <= ky_hi; ky++) {
            const int yy = y + ky;
            __syncthreads();  // previous tap row fully consumed
            // cost rows, wrapped columns (seq/AdaptiveWeightAggregation.cpp:95-97); real pixels
            // wrap once (r < W), columns of padding pixels past the image end are clamped
            const size_t crow = (size_t)yy * W;
            if (vec) {
                for (int q = tid; q < (kAwTX + 2 * r) * (kAwDC / 4); q += kAwThreads) {
                    const int xi = q >> 4, d4 = (q & 15) * 4;
                    const int xs = imin(imax(wrap1(x0 - r + xi, W), 0), W - 1);
                    const int dg = dc0 + d4;
                    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (dg < D) {
                        const CT *src = vol + (crow + xs) * D + dg;
                        if constexpr (sizeof(CT) == 4) {
                            v = *reinterpret_cast<const float4 *>(src);
                        } else {
                            const uint2 hv = *reinterpret_cast<const uint2 *>(src);
                            const float2 f0 = __half22float2(*reinterpret_cast<const __half2 *>(&hv.x));
                            const float2 f1 = __half22float2(*reinterpret_cast<const __half2 *>(&hv.y));
                            v = make_float4(f0.x, f0.y, f1.x, f1.y);
                        }
                    }
                    *reinterpret_cast<float4 *>(Cs + xi * kAwCPitch + d4) = v;
                }
            } else {
                for (int q = tid; q < (kAwTX + 2 * r) * kAwDC; q += kAwThreads) {
                    const int xi = q >> 6, dd = q & 63;
                    const int xs = imin(imax(wrap1(x0 - r + xi, W), 0), W - 1);
                    const int dg = dc0 + dd;
                    Cs[xi * kAwCPitch + dd] = (dg < D) ? to_f32(vol[(crow + xs) * D + dg]) : 0.f;
                }
            }
            // packed Lab of the tap row: reference columns x0-r .., target columns tbase-r ..
            for (int q = tid; q < kAwTX + 2 * r; q += kAwThreads) {
                const int xc = x0 - r + q;
                labRrow[q] = (xc >= 0 && xc < W) ? labr[crow + xc] : kLabOut;
            }
            for (int q = tid; q < NT + 2 * r; q += kAwThreads) {
                const int xc = tbase - r + q;
                labTrow[q] = (xc >= 0 && xc < W) ? labt[crow + xc] : kLabOut;
            }
            __syncthreads();
            const float *pwrow = pw + (ky + r) * e;
            // weights of two taps per pass (kx and kx + 8), the table reads of both in
            // flight together: the colour-distance index of every weight first, then the
            // reads, then the products
            for (int kx = warp; kx < e; kx += 2 * (kAwThreads / 32)) {
                uint32_t idx[2][6];
                bool ok[2][6];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int k = kx + h * (kAwThreads / 32);
#pragma unroll
                    for (int m = 0; m < 2; m++) {
                        const uint32_t q = labRrow[imin(lane + 32 * m + k, kAwTX + 2 * r - 1)];
                        ok[h][m] = k < e && !((q | cR[m]) & kLabOut);
                        const uint32_t ad = __vabsdiffu4(cR[m], q);
                        idx[h][m] = __dp4a(ad, ad, 0u);
                    }
#pragma unroll
                    for (int m = 0; m < 4; m++) {
                        const int u = lane + 32 * m;
                        uint32_t q = labTrow[imin(u + k, NT + 2 * r - 1)];
                        if (wrapped_tile && tbase + u < 0 && k < e) {
                            // the target column is t + W: its tap is column t + W + k - r
                            const int xc = tbase + u + W + k - r;
                            q = (xc >= 0 && xc < W) ? labt[crow + xc] : kLabOut;
                        }
                        ok[h][2 + m] = k < e && u < NT && !((q | cT[m]) & kLabOut);
                        const uint32_t ad = __vabsdiffu4(cT[m], q);
                        idx[h][2 + m] = __dp4a(ad, ad, 0u);
                    }
                }
                float g[2][6];
#pragma unroll
                for (int h = 0; h < 2; h++)
#pragma unroll
                    for (int m = 0; m < 6; m++) g[h][m] = ok[h][m] ? __ldg(G + idx[h][m]) : 0.f;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int k = kx + h * (kAwThreads / 32);
                    if (k < e) {
                        // seq/AdaptiveWeightAggregation.cpp:33-71: pw[k] * expf(-dist / gamma_s),
                        // 0 where the tap (or a padding centre) is outside the image
                        const float pwk = __ldg(pwrow + k);
#pragma unroll
                        for (int m = 0; m < 2; m++) wRs[k * kAwTX + lane + 32 * m] = ok[h][m] ? __fmul_rn(pwk, g[h][m]) : 0.f;
#pragma unroll
                        for (int m = 0; m < 4; m++) {
                            const int u = lane + 32 * m;
                            if (u < NT) wTs[k * NTP + u] = ok[h][2 + m] ? __fmul_rn(pwk, g[h][2 + m]) : 0.f;
                        }
                    }
                }
            }
            __syncthreads();

            // u index of wT for (j, i): px0 + j - 4td - i + 63 = ubase + (j - i) + 3
            const int ubase = px0 - 4 * td + kAwDC - 4;
            const float *cp = Cs + px0 * kAwCPitch + 4 * td;  // cost column px0 + kx, + kx * pitch
            const float *wrp = wRs + px0;                      // + kx * 64
            const float *wtp = wTs + ubase;                    // + kx * NTP
            // one tap: 4 pixels x 4 disparities, reference order per entry
            auto tap = [&](const float (*cw)[4], int cofs, const float *wr4, const float *wt7) {
                float wr[4], wt[7];
                const float4 a0 = *reinterpret_cast<const float4 *>(wr4);
                wr[0] = a0.x; wr[1] = a0.y; wr[2] = a0.z; wr[3] = a0.w;
                const float4 b0 = *reinterpret_cast<const float4 *>(wt7);
                const float4 b1 = *reinterpret_cast<const float4 *>(wt7 + 4);
                wt[0] = b0.x; wt[1] = b0.y; wt[2] = b0.z; wt[3] = b0.w;
                wt[4] = b1.x; wt[5] = b1.y; wt[6] = b1.z;
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        // w of disparities i = 2h, 2h+1: wR * wT (index j - i + 3)
                        const unsigned long long w = pack2(__fmul_rn(wr[j], wt[j - 2 * h + 3]),
                                                           __fmul_rn(wr[j], wt[j - 2 * h + 2]));
                        const unsigned long long c = pack2(cw[j + cofs][2 * h], cw[j + cofs][2 * h + 1]);
                        sw[j][h] = add2(sw[j][h], w);
                        if constexpr (EXACT) sc[j][h] = add2(sc[j][h], mul2(c, w));
                        else sc[j][h] = fma2(c, w, sc[j][h]);
                    }
            };
            int kx = 0;
            // taps in groups of 4: the 7 cost columns px0+kx .. px0+kx+6 of a group are
            // loaded once and serve 4 pixels x 4 taps
#pragma unroll 1
            for (; kx + 4 <= e; kx += 4, cp += 4 * kAwCPitch, wrp += 4 * kAwTX, wtp += 4 * NTP) {
                float cw[7][4];
#pragma unroll
                for (int q = 0; q < 7; q++) {
                    const float4 v = *reinterpret_cast<const float4 *>(cp + q * kAwCPitch);
                    cw[q][0] = v.x; cw[q][1] = v.y; cw[q][2] = v.z; cw[q][3] = v.w;
                }
#pragma unroll
                for (int u = 0; u < 4; u++) tap(cw, u, wrp + u * kAwTX, wtp + u * NTP);
            }
#pragma unroll 1
            for (; kx < e; kx++, cp += kAwCPitch, wrp += kAwTX, wtp += NTP) {
                float cw[4][4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float4 v = *reinterpret_cast<const float4 *>(cp + q * kAwCPitch);
                    cw[q][0] = v.x; cw[q][1] = v.y; cw[q][2] = v.z; cw[q][3] = v.w;
                }
                tap(cw, 0, wrp, wtp);
            }
        }
        __syncthreads();
        // score / sum of weights (seq/AdaptiveWeightAggregation.cpp:108), staged for the arg-min
        float *outs = Cs;  // [64][kAwDC + 1]
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float v = __fdiv_rn(half2_of(sc[j][i >> 1], i & 1), half2_of(sw[j][i >> 1], i & 1));
                outs[(px0 + j) * (kAwDC + 1) + 4 * td + i] = v;
                const int x = x0 + px0 + j, dg = dc0 + 4 * td + i;
                if (cost_out && x < W && dg < D) cost_out[((size_t)y * W + x) * D + dg] = v;
            }
        __syncthreads();
        if (tid < kAwTX) {
            float bv = best_v[tid];
            int bx = best_i[tid];
            const int nd = imin(kAwDC, D - dc0);
            for (int dd = 0; dd < nd; dd++) {
                const float v = outs[tid * (kAwDC + 1) + dd];
                if (v < bv) {  // first strict minimum in increasing d
                    bv = v;
                    bx = dc0 + dd;
                }
            }
            best_v[tid] = bv;
            best_i[tid] = bx;
        }
    }
    if (tid < kAwTX && x0 + tid < W) {
        const int x = x0 + tid;
        const bool found = best_i[tid] != 0;
        raw[(size_t)y * W + x] = found ? (uint16_t)(0x100 | best_i[tid]) : (uint16_t)0;
        if (found) atomicMax(row_last + y, x);
    }
}

// ---------------------------------------------------------------------------
// k_aw_wta, software-pipelined over the tap rows: while the
// block adds tap row ky, the cost rows of ky + 1 arrive by cp.async in the
// other buffer, the weights of ky + 1 are made in slices between the groups of
// taps (their table reads in flight across a group), and the Lab rows of
// ky + 2 are staged; one barrier per tap row.  The arithmetic per entry is
// k_aw_wta's: EXACT (plain form, f32 volume) the reference's order, unfused;
// otherwise (FP16 form, f16 volume staged as f16, D a multiple of 8) one FMA.
// E: the window edge as a constant (33, the reference driver's 33 x 33 window), so
// that the tap loop unrolls whole, or 0 for the edge of the e argument.
__device__ int g_aw_tma_timeouts;
uint64_t aw_tma_timeouts() {
    int v = 0;
    return cudaMemcpyFromSymbol(&v, g_aw_tma_timeouts, sizeof(int)) == cudaSuccess ? (uint64_t)v : 0;
}

template <typename CT, bool EXACT, int E>
__global__ void __launch_bounds__(kAwThreads, 2) k_aw_wta_pipe(const __grid_constant__ CUtensorMap tmap, int use_tma,
                                                          const CT *__restrict__ vol,
                                                          const uint32_t *__restrict__ labr,
                                                          const uint32_t *__restrict__ labt,
                                                          const float *__restrict__ pw, const float *__restrict__ G,
                                                          uint16_t *__restrict__ raw, int *__restrict__ row_last,
                                                          float *__restrict__ cost_out, int H, int W, int D, int e_arg,
                                                          float zero) {
    const int e = E ? E : e_arg;
    const int r = e >> 1;
    // zero: +0.0f from the host.  A packed multiply whose result feeds a packed add is
    // contracted into one fused multiply-add by the compiler, even written as
    // mul.rn / __fmul2_rn; a fused multiply-add with this zero as its addend (which
    // the compiler cannot know is zero) rounds like the multiply alone and is not
    // fused further, so the plain form's products C*w stay IEEE products, two to an
    // instruction.
    const float2 z2 = make_float2(zero, zero);
    constexpr int NT = kAwTX + kAwDC - 1;  // target columns of a tile
    constexpr int NTP = NT + 1;
    // cost rows: 64 floats (dense, as a TMA copy writes them), or kAwHPitch halves
    // (16-byte rows for the copies, the pitch keeping a half warp's rows apart in banks)
    constexpr int CP = sizeof(CT) == 4 ? kAwDC : kAwHPitch;
    const int CS = (kAwTX + 2 * r + 4) * CP * (int)sizeof(CT) / 4;  // floats of one cost buffer
    // no static shared memory: the dynamic buffers begin at the block's shared base,
    // which the TMA copies need 128-byte aligned (checked per block; blocks whose
    // base is not take cp.async).  The declaration promises only 16 bytes, the
    // alignment the compiler's address arithmetic was tuned under.
    extern __shared__ __align__(16) float psm_[];
    // buffer b: costs at psm_ + b CS, reference weights at wR0 + b e 64, target weights at wT0 + b e NTP
    float *const wR0 = psm_ + 2 * CS, *const wT0 = wR0 + 2 * e * kAwTX;
    uint32_t *labbase = reinterpret_cast<uint32_t *>(psm_ + 2 * CS + 2 * e * kAwTX + 2 * e * NTP);
    const int LRN = kAwTX + 2 * r, LTN = NT + 2 * r;  // words of a reference / target Lab row
    float *const best_v = reinterpret_cast<float *>(labbase + 3 * (LRN + LTN));  // [kAwTX]
    int *const best_i = reinterpret_cast<int *>(best_v + kAwTX);                  // [kAwTX]
    // plain form, tiles whose cost columns need no wrap: each tap row's cost rows arrive
    // by one TMA copy (box 64 disparities x (64 + 2r) columns) completing on cbar[buffer]
    uint64_t *const cbar =
        reinterpret_cast<uint64_t *>((reinterpret_cast<uintptr_t>(best_i + kAwTX) + 7) & ~uintptr_t(7));  // [2]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = kAwThreads / 32;
    // tap tile: warp (wx, wd) = (warp & 3, warp >> 2) takes pixels 16 wx .. 16 wx + 15 and
    // disparities 32 wd .. 32 wd + 31 of the tile; lane (pg, dg) = (lane >> 3, lane & 7)
    // four pixels px0 .. px0+3 and four disparities dd0 .. dd0+3 of those.  Per tap a
    // warp reads 4 distinct reference weights, 11 distinct 16-byte target-weight
    // runs and one new cost column of 32 x 4 values (the other three of a thread's
    // window are in registers from the previous taps).
    const int px0 = 16 * (warp & 3) + 4 * (lane >> 3);
    const int dd0 = 32 * (warp >> 2) + 4 * (lane & 7);
    const int y = blockIdx.y, x0 = blockIdx.x * kAwTX;
    if (tid < kAwTX) {
        best_v[tid] = __int_as_float(0x7f800000);
        best_i[tid] = 0x7fffffff;
    }
    const bool vec = (D & 3) == 0;
    const bool tma_tile = sizeof(CT) == 4 && use_tma && x0 - r >= 0 && x0 + kAwTX + r <= W &&
                          ((uint32_t)__cvta_generic_to_shared(psm_) & 127) == 0;
    const uint32_t cb0 = (uint32_t)__cvta_generic_to_shared(cbar);
    uint32_t cphase = 0;  // bit b: parity of the next completion of cbar[b]
    if (tma_tile && tid == 0) {
        mbar_init(cb0);
        mbar_init(cb0 + 8);
    }
    // (the barriers' initialisation is published by the chunk loop's first __syncthreads)
    auto cost_wait = [&](int b) {
        if (!tma_tile) return;
        if (!mbar_wait(cb0 + 8 * b, (cphase >> b) & 1)) {
            if (tid == 0) atomicAdd(&g_aw_tma_timeouts, 1);
            mbar_wait(cb0 + 8 * b, (cphase >> b) & 1);  // the copy may still land in this buffer
        }
        cphase ^= 1u << b;
    };

    for (int dc0 = 0; dc0 < D; dc0 += kAwDC) {
        // sums of disparity pairs (dd0 + 2h, dd0 + 2h + 1) of pixel px0 + j, as float2 for
        // the packed adds (each half an IEEE round-to-nearest operation)
        float2 sw[4][2], sc[4][2];
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int h = 0; h < 2; h++) sw[j][h] = sc[j][h] = make_float2(0.f, 0.f);
        const int tbase = x0 - dc0 - (kAwDC - 1);
        uint32_t cR[2], cT[4];
#pragma unroll
        for (int m = 0; m < 2; m++) {
            const int x = x0 + lane + 32 * m;
            cR[m] = x < W ? labr[(size_t)y * W + x] : kLabOut;
        }
#pragma unroll
        for (int m = 0; m < 4; m++) {
            int t = tbase + lane + 32 * m;
            if (t < 0) t += W;  // seq/AdaptiveWeightAggregation.cpp:87
            cT[m] = (lane + 32 * m < NT && t >= 0 && t < W) ? labt[(size_t)y * W + t] : kLabOut;
        }
        const bool wrapped_tile = tbase < 0;
        const int ky_lo = imax(-r, -y), ky_hi = imin(r, H - 1 - y);

        // cost rows of tap row ky into C by cp.async (zero fill past D); wrapped
        // columns as in k_aw_wta (seq/AdaptiveWeightAggregation.cpp:95-97)
        auto stage_cost = [&](int ky, int b) {
            float *C = psm_ + b * CS;
            const size_t crow = (size_t)(y + ky) * W;
            const uint32_t cbase = (uint32_t)__cvta_generic_to_shared(C);
            if (tma_tile) {
                if (tid == 0)
                    tma_load_3d(cbase, &tmap, dc0, x0 - r, y + ky, cb0 + 8 * b,
                                (uint32_t)((kAwTX + 2 * r) * kAwDC * sizeof(float)));
                return;
            }
            if constexpr (sizeof(CT) == 2) {
                // f16 volume: 16-byte copies of 8 disparities (D is a multiple of 8)
                for (int q = tid; q < (kAwTX + 2 * r) * (kAwDC / 8); q += kAwThreads) {
                    const int xi = q >> 3, d8 = (q & 7) * 8;
                    const int xs = imin(imax(wrap1(x0 - r + xi, W), 0), W - 1);
                    const int dg = dc0 + d8;
                    const CT *src = vol + (crow + xs) * D + (dg < D ? dg : 0);
                    const uint32_t dst = cbase + (uint32_t)((xi * CP + d8) * 2);
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
                                 "r"(dg < D ? 16 : 0)
                                 : "memory");
                }
            } else if (vec) {
                for (int q = tid; q < (kAwTX + 2 * r) * (kAwDC / 4); q += kAwThreads) {
                    const int xi = q >> 4, d4 = (q & 15) * 4;
                    const int xs = imin(imax(wrap1(x0 - r + xi, W), 0), W - 1);
                    const int dg = dc0 + d4;
                    const float *src = vol + (crow + xs) * D + (dg < D ? dg : 0);
                    const uint32_t dst = cbase + (uint32_t)((xi * CP + d4) * 4);
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
                                 "r"(dg < D ? 16 : 0)
                                 : "memory");
                }
            } else {
                for (int q = tid; q < (kAwTX + 2 * r) * kAwDC; q += kAwThreads) {
                    const int xi = q >> 6, dd = q & 63;
                    const int xs = imin(imax(wrap1(x0 - r + xi, W), 0), W - 1);
                    const int dg = dc0 + dd;
                    const float *src = vol + (crow + xs) * D + (dg < D ? dg : 0);
                    const uint32_t dst = cbase + (uint32_t)((xi * CP + dd) * 4);
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(src),
                                 "r"(dg < D ? 4 : 0)
                                 : "memory");
                }
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        };
        auto stage_lab = [&](int ky, int slot) {
            const size_t crow = (size_t)(y + ky) * W;
            uint32_t *LR = labbase + slot * (LRN + LTN), *LT = LR + LRN;
            for (int q = tid; q < LRN; q += kAwThreads) {
                const int xc = x0 - r + q;
                LR[q] = (xc >= 0 && xc < W) ? labr[crow + xc] : kLabOut;
            }
            for (int q = tid; q < LTN; q += kAwThreads) {
                const int xc = tbase - r + q;
                LT[q] = (xc >= 0 && xc < W) ? labt[crow + xc] : kLabOut;
            }
        };
        // weights of tap (ky, k) for this warp's lanes, in two halves: the table
        // indices and reads (issue), then the products (finish)
        struct Slice {
            uint32_t idx[6];
            bool ok[6];
            float g[6];
        };
        // (every caller passes k < e, so the reference index lane + 32 m + k <= 63 + 2r
        // stays inside its row, and the target index u + k only passes the row's end
        // for u = 127, the padding target of lane 31)
        auto slice_issue = [&](Slice &sl, int ky, int k, int slot) {
            const uint32_t *LR = labbase + slot * (LRN + LTN), *LT = LR + LRN;
#pragma unroll
            for (int m = 0; m < 2; m++) {
                const uint32_t q = LR[lane + 32 * m + k];
                sl.ok[m] = !((q | cR[m]) & kLabOut);
                const uint32_t ad = __vabsdiffu4(cR[m], q);
                sl.idx[m] = __dp4a(ad, ad, 0u);
            }
            uint32_t qt[4];
#pragma unroll
            for (int m = 0; m < 3; m++) qt[m] = LT[lane + 32 * m + k];
            qt[3] = LT[imin(lane + 96 + k, LTN - 1)];
            if (wrapped_tile) {
                // targets that wrapped around the left edge: their taps come from the
                // other end of the row (block-uniform branch)
                const size_t crow = (size_t)(y + ky) * W;
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    const int u = lane + 32 * m;
                    if (tbase + u < 0) {
                        const int xc = tbase + u + W + k - r;
                        qt[m] = (xc >= 0 && xc < W) ? labt[crow + xc] : kLabOut;
                    }
                }
            }
#pragma unroll
            for (int m = 0; m < 4; m++) {
                sl.ok[2 + m] = (m < 3 || lane < 31) && !((qt[m] | cT[m]) & kLabOut);
                const uint32_t ad = __vabsdiffu4(cT[m], qt[m]);
                sl.idx[2 + m] = __dp4a(ad, ad, 0u);
            }
#pragma unroll
            for (int m = 0; m < 6; m++) sl.g[m] = sl.ok[m] ? __ldg(G + sl.idx[m]) : 0.f;
        };
        auto slice_finish = [&](const Slice &sl, int ky, int k, float *wR, float *wT) {
            if (k < e) {
                // seq/AdaptiveWeightAggregation.cpp:33-71: pw[k] * expf(-dist / gamma_s)
                const float pwk = __ldg(pw + (ky + r) * e + k);
#pragma unroll
                for (int m = 0; m < 2; m++) wR[k * kAwTX + lane + 32 * m] = sl.ok[m] ? __fmul_rn(pwk, sl.g[m]) : 0.f;
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    const int u = lane + 32 * m;
                    if (u < NT) wT[k * NTP + u] = sl.ok[2 + m] ? __fmul_rn(pwk, sl.g[2 + m]) : 0.f;
                }
            }
        };

        // prologue: Lab rows of the first two tap rows, costs and weights of the first
        __syncthreads();  // the previous chunk is done with every buffer
        stage_lab(ky_lo, 0);
        if (ky_lo + 1 <= ky_hi) stage_lab(ky_lo + 1, 1);
        stage_cost(ky_lo, 0);
        __syncthreads();
        for (int k = warp; k < e; k += NW) {
            Slice sl;
            slice_issue(sl, ky_lo, k, 0);
            slice_finish(sl, ky_lo, k, wR0, wT0);
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        cost_wait(0);
        __syncthreads();

        for (int ky = ky_lo; ky <= ky_hi; ky++) {
            const int i = ky - ky_lo, b = i & 1;
            const bool next = ky + 1 <= ky_hi;
            if (next) stage_cost(ky + 1, b ^ 1);
            if (ky + 2 <= ky_hi) stage_lab(ky + 2, (i + 2) % 3);
            const int lnext = (i + 1) % 3;
            const float *Cs = psm_ + b * CS, *wRs = wR0 + b * e * kAwTX, *wTs = wT0 + b * e * NTP;
            float *wRn = wR0 + (b ^ 1) * e * kAwTX, *wTn = wT0 + (b ^ 1) * e * NTP;

            // target weights of entry (j, i): u = px0 + j - (dd0 + i) + 63, so a thread's
            // seven are ub .. ub+6 (the eighth loaded is ub+7 <= 127, inside the row)
            const int ub = px0 - dd0 + kAwDC - 4;
            const CT *cp = reinterpret_cast<const CT *>(Cs) + px0 * CP + dd0;  // staged column px0 + kx
            const float *wrp = wRs + px0;
            const float *wtp = wTs + ub;
            // four disparities of a staged cost column as floats
            auto col4 = [&](const CT *q, float *o) {
                if constexpr (sizeof(CT) == 4) {
                    const float4 v = *reinterpret_cast<const float4 *>(q);
                    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
                } else {
                    const uint2 hv = *reinterpret_cast<const uint2 *>(q);
                    const float2 f0 = __half22float2(*reinterpret_cast<const __half2 *>(&hv.x));
                    const float2 f1 = __half22float2(*reinterpret_cast<const __half2 *>(&hv.y));
                    o[0] = f0.x; o[1] = f0.y; o[2] = f1.x; o[3] = f1.y;
                }
            };
            // one tap over the thread's 4 pixels x 4 disparities; cw[j] is the cost column
            // of pixel j at this tap.  Plain form (EXACT): w = wR*wT, sw += w, sc += C*w, each
            // an IEEE operation (seq/AdaptiveWeightAggregation.cpp:100-103): w by scalar
            // multiplies, C*w by the packed multiply-add with the opaque zero, the sums by
            // packed adds.  FP16 form: sc = fma(C, w, sc).
            auto tap = [&](const float (&cw)[4][4], const float *wr4, const float *wt8) {
                float wr[4], wt[8];
                const float4 a0 = *reinterpret_cast<const float4 *>(wr4);
                wr[0] = a0.x; wr[1] = a0.y; wr[2] = a0.z; wr[3] = a0.w;
                const float4 b0 = *reinterpret_cast<const float4 *>(wt8);
                const float4 b1 = *reinterpret_cast<const float4 *>(wt8 + 4);
                wt[0] = b0.x; wt[1] = b0.y; wt[2] = b0.z; wt[3] = b0.w;
                wt[4] = b1.x; wt[5] = b1.y; wt[6] = b1.z; wt[7] = b1.w;
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const float w0 = __fmul_rn(wr[j], wt[j - 2 * h + 3]);
                        const float w1 = __fmul_rn(wr[j], wt[j - 2 * h + 2]);
                        sw[j][h] = __fadd2_rn(sw[j][h], make_float2(w0, w1));
                        if constexpr (EXACT)
                            sc[j][h] = __fadd2_rn(sc[j][h], __ffma2_rn(make_float2(cw[j][2 * h], cw[j][2 * h + 1]),
                                                                       make_float2(w0, w1), z2));
                        else
                            sc[j][h] = __ffma2_rn(make_float2(cw[j][2 * h], cw[j][2 * h + 1]), make_float2(w0, w1),
                                                  sc[j][h]);
                    }
            };
            // the cost window slides one column per tap: win holds columns kx .. kx+2 of
            // the thread's first pixel, each tap adds column kx+3
            float win[3][4];
#pragma unroll
            for (int q = 0; q < 3; q++) col4(cp + q * CP, win[q]);
            int kx = 0, sj = 0;
#pragma unroll(E ? 8 : 1)
            for (; kx + 4 <= e; kx += 4, sj++) {
                // a slice of the next tap row's weights around this group of taps
                const int ks = warp + NW * sj;
                const bool dos = next && ks < e;
                Slice sl;
                if (dos) slice_issue(sl, ky + 1, ks, lnext);
                float nc[4][4];
#pragma unroll
                for (int u = 0; u < 4; u++) col4(cp + (kx + 3 + u) * CP, nc[u]);
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    float cw[4][4];
#pragma unroll
                    for (int j = 0; j < 4; j++)
#pragma unroll
                        for (int i = 0; i < 4; i++) cw[j][i] = (u + j < 3) ? win[u + j][i] : nc[u + j - 3][i];
                    tap(cw, wrp + (kx + u) * kAwTX, wtp + (kx + u) * NTP);
                }
#pragma unroll
                for (int q = 0; q < 3; q++)
#pragma unroll
                    for (int i = 0; i < 4; i++) win[q][i] = nc[q + 1][i];
                if (dos) slice_finish(sl, ky + 1, ks, wRn, wTn);
            }
#pragma unroll(E ? 3 : 1)
            for (; kx < e; kx++) {
                float cw[4][4];
                col4(cp + (kx + 3) * CP, cw[3]);
#pragma unroll
                for (int q = 0; q < 3; q++)
#pragma unroll
                    for (int i = 0; i < 4; i++) cw[q][i] = win[q][i];
                tap(cw, wrp + kx * kAwTX, wtp + kx * NTP);
#pragma unroll
                for (int q = 0; q < 3; q++)
#pragma unroll
                    for (int i = 0; i < 4; i++) win[q][i] = cw[q + 1][i];
            }
            // slices the groups did not reach (short windows)
            if (next)
                for (int ks = warp + NW * sj; ks < e; ks += NW) {
                    Slice sl;
                    slice_issue(sl, ky + 1, ks, lnext);
                    slice_finish(sl, ky + 1, ks, wRn, wTn);
                }
            asm volatile("cp.async.wait_all;\n" ::: "memory");
            if (next) cost_wait(b ^ 1);
            __syncthreads();
        }
        // score / sum of weights (seq/AdaptiveWeightAggregation.cpp:108), staged for the arg-min
        float *outs = psm_;  // [64][kAwDC + 1]
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float2 a2 = sc[j][i >> 1], b2 = sw[j][i >> 1];
                const float v = __fdiv_rn((i & 1) ? a2.y : a2.x, (i & 1) ? b2.y : b2.x);
                outs[(px0 + j) * (kAwDC + 1) + dd0 + i] = v;
                const int x = x0 + px0 + j, dg = dc0 + dd0 + i;
                if (cost_out && x < W && dg < D) cost_out[((size_t)y * W + x) * D + dg] = v;
            }
        __syncthreads();
        if (tid < kAwTX) {
            float bv = best_v[tid];
            int bx = best_i[tid];
            const int nd = imin(kAwDC, D - dc0);
            for (int dd = 0; dd < nd; dd++) {
                const float v = outs[tid * (kAwDC + 1) + dd];
                if (v < bv) {  // first strict minimum in increasing d
                    bv = v;
                    bx = dc0 + dd;
                }
            }
            best_v[tid] = bv;
            best_i[tid] = bx;
        }
    }
    if (tid < kAwTX && x0 + tid < W) {
        const int x = x0 + tid;
        const bool found = best_i[tid] != 0;
        raw[(size_t)y * W + x] = found ? (uint16_t)(0x100 | best_i[tid]) : (uint16_t)0;
        if (found) atomicMax(row_last + y, x);
    }
}

// ---------------------------------------------------------------------------
// host orchestration

static bool fast_kind(int k) { return k == RTS_COST_AD || k == RTS_COST_CENSUS; }

bool fast_costs(const rts_params &p) {
    if (!fast_kind(p.cost1) || !(p.cost2 == RTS_COST_NONE || fast_kind(p.cost2))) return false;
    const bool census = p.cost1 == RTS_COST_CENSUS || p.cost2 == RTS_COST_CENSUS;
    return !census || (2 * p.census_hrad + 1) * (2 * p.census_wrad + 1) <= 64;
}

bool fused_supported(const rts_params &p, int H, int W) {
    (void)H;
    (void)W;
    if (p.aggr == RTS_AGGR_CROSS) return cross_fused_supported(p);
    if (p.aggr == RTS_AGGR_AW) return p.aw_rad <= 16;
    return false;
}

rts_status prep_records(rts_ctx *c, const rts_params &p, int H, int W, const uint8_t *gray, const uint8_t *rgb,
                        uint4 *rec, uint32_t *arms_out) {
    const bool code = p.cost1 == RTS_COST_CENSUS || p.cost2 == RTS_COST_CENSUS;
    const bool arms = p.aggr == RTS_AGGR_CROSS;
    k_prep_records<<<dim3((W + 127) / 128, H), 128, 0, c->stream>>>(gray, rgb, rec, arms_out, H, W, p.census_hrad,
                                                                   p.census_wrad, p.cross_arm, p.cross_tau,
                                                                   code && fast_costs(p), arms);
    count_launch(c);
    return check_launch(c, "prep_records");
}

static rts_status cost_cfg(rts_ctx *c, const rts_params &p, CostCfg *cfg) {
    cfg->k1 = p.cost1;
    cfg->k2 = p.cost2;
    cfg->trunc1 = (p.cost1 == RTS_COST_AD && p.aggr == RTS_AGGR_CROSS) ? 1 : 0;  // seq/Main.cpp:183-186
    cfg->trunc = p.ad_trunc;
    cfg->l1 = p.lambda1;
    cfg->l2 = p.lambda2;
    cfg->lut1 = cfg->lut2 = nullptr;
    // integer fast path: AD with an integral truncation (or none) and census take
    // integer values below the table size (AD <= 765, census <= 64)
    const bool trunc_ok = !cfg->trunc1 || (p.ad_trunc >= 0.f && p.ad_trunc < (float)kCombineLut &&
                                          p.ad_trunc == floorf(p.ad_trunc));
    cfg->int_path = trunc_ok ? 1 : 0;
    cfg->itrunc = cfg->trunc1 ? (int)p.ad_trunc : 0x7fffffff;
    if (p.cost2 != RTS_COST_NONE) return combine_luts(c, p.lambda1, p.lambda2, &cfg->lut1, &cfg->lut2);
    return RTS_OK;
}

rts_status cost_volume_fast(rts_ctx *c, const rts_params &p, int H, int W, const uint4 *rr, const uint4 *rt,
                            void *vol, int half) {
    CostCfg cfg;
    RTS_TRY(cost_cfg(c, p, &cfg));
    const int D = p.disp_range;
    if (cfg.int_path && cfg.k1 == RTS_COST_AD && cfg.k2 == RTS_COST_CENSUS) {
        const dim3 g((unsigned)((W + kAdcTX - 1) / kAdcTX), H);
        if (half) k_cost_volume_adc<__half><<<g, 256, 0, c->stream>>>(rr, rt, (__half *)vol, H, W, D, cfg.itrunc, cfg.lut1, cfg.lut2);
        else k_cost_volume_adc<float><<<g, 256, 0, c->stream>>>(rr, rt, (float *)vol, H, W, D, cfg.itrunc, cfg.lut1, cfg.lut2);
        count_launch(c);
        return check_launch(c, "cost_volume");
    }
    const dim3 g((unsigned)(((long)W * D + 255) / 256), H);
    if (half) k_cost_volume<__half><<<g, 256, 0, c->stream>>>(rr, rt, (__half *)vol, H, W, D, cfg);
    else k_cost_volume<float><<<g, 256, 0, c->stream>>>(rr, rt, (float *)vol, H, W, D, cfg);
    count_launch(c);
    return check_launch(c, "cost_volume");
}

bool cross_fused_supported(const rts_params &p) {
    // 16-byte row copies in the vertical kernel need D a multiple of 8; the
    // 64-entry ring of the horizontal kernel bounds the arm length (k_batch.cu)
    return p.cross_arm <= 23 && p.disp_range % 8 == 0;
}

rts_status aw_fused(rts_ctx *c, const rts_params &p, int H, int W, const void *vol, int half, const uint8_t *labr,
                    const uint8_t *labt, uint16_t *raw, int *rl, float *cost_out) {
    const float *pw, *g;
    RTS_TRY(prox_weights(c, p.aw_gamma_p, p.aw_rad, &pw));
    RTS_TRY(lab_weight_lut(c, p.aw_gamma_s, &g));
    const long np = (long)H * W;
    void *lp;
    RTS_TRY(scratch(c, SL_V_MEAN, (size_t)np * 8, &lp));
    uint32_t *plr = (uint32_t *)lp, *plt = plr + np;
    k_pack_lab<<<(unsigned)((np + 255) / 256), 256, 0, c->stream>>>(labr, plr, np);
    k_pack_lab<<<(unsigned)((np + 255) / 256), 256, 0, c->stream>>>(labt, plt, np);
    count_launch(c, 2);
    const int r = p.aw_rad, e = 2 * r + 1;
    const size_t smem = sizeof(float) * ((size_t)(kAwTX + 2 * r + 4) * kAwCPitch + (size_t)e * kAwTX +
                                         (size_t)e * (kAwTX + kAwDC) + (size_t)(kAwTX + 2 * r) +
                                         (size_t)(kAwTX + kAwDC - 1 + 2 * r));
    const dim3 grid((W + kAwTX - 1) / kAwTX, H);
    StageScope sc(c, "aw_wta");
    auto go = [&](auto kern, auto *v) -> rts_status {
        RTS_TRY(set_smem(c, kern, smem, "aw_wta"));
        kern<<<grid, kAwThreads, smem, c->stream>>>(v, plr, plt, pw, g, raw, rl, cost_out, H, W, p.disp_range, e);
        return RTS_OK;
    };
    // plain form: bit-exact float volume, the pipelined kernel; FP16 form: __half
    // volume and fused multiply-add
    // the pipelined kernel: two cost buffers (f32 rows, or f16 rows of 8-disparity
    // copies; their space also holds the [64][65] argmin staging), two weight
    // buffers, three Lab row pairs
    // two cost buffers (their space also holds the [64][65] arg-min staging), two
    // weight buffers, three Lab row pairs, the arg-min state and two mbarriers
    auto pipe_smem = [&](size_t row_bytes) {
        const size_t costs = 2 * (size_t)(kAwTX + 2 * r + 4) * row_bytes;
        return std::max(costs, (size_t)kAwTX * (kAwDC + 1) * 4) +
               sizeof(float) * (2 * (size_t)e * kAwTX + 2 * (size_t)e * (kAwTX + kAwDC)) +
               sizeof(uint32_t) * 3 * ((size_t)(kAwTX + 2 * r) + (size_t)(kAwTX + kAwDC - 1 + 2 * r)) +
               2 * kAwTX * 4 + 24;
    };
    CUtensorMap tm{};
    if (half && p.disp_range % 8 != 0) {
        RTS_TRY(go(k_aw_wta<__half, false>, (const __half *)vol));
    } else if (half) {
        const size_t psmem = pipe_smem((size_t)kAwHPitch * 2);
        auto kern = e == 33 ? k_aw_wta_pipe<__half, false, 33> : k_aw_wta_pipe<__half, false, 0>;
        RTS_TRY(set_smem(c, kern, psmem, "aw_wta_pipe"));
        kern<<<grid, kAwThreads, psmem, c->stream>>>(tm, 0, (const __half *)vol, plr, plt, pw, g, raw, rl, cost_out,
                                                     H, W, p.disp_range, e, 0.f);
    } else {
        // dense 64-float cost rows; the tiles whose columns need no wrap take them by TMA
        const size_t psmem = pipe_smem((size_t)kAwDC * 4);
        const int use_tma = volume_tensor_map(&tm, vol, H, W, p.disp_range, 4, kAwDC, kAwTX + 2 * r, 1) ? 1 : 0;
        auto kern = e == 33 ? k_aw_wta_pipe<float, true, 33> : k_aw_wta_pipe<float, true, 0>;
        RTS_TRY(set_smem(c, kern, psmem, "aw_wta_pipe"));
        kern<<<grid, kAwThreads, psmem, c->stream>>>(tm, use_tma, (const float *)vol, plr, plt, pw, g, raw, rl,
                                                     cost_out, H, W, p.disp_range, e, 0.f);
    }
    count_launch(c);
    return check_launch(c, "aw_wta");
}

}  // namespace rts
