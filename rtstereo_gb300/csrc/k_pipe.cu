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
//   k_cross_hseg    cost -> running sum along x (seq/CrossBasedAggregation.cpp:117-125)
//                   -> row segment P[x+r]-P[x-l-1] (:151-160), one warp per
//                   (row, 32 disparities), running sums kept in a shared-memory ring
//   k_cross_vert    vertical sum of row segments / pixel count (:140-167) and the
//                   first strict arg-min over d (seq/WTA.cpp:15-22), one warp per
//                   (column, 32 disparities), segments kept in a shared-memory ring
//   k_aw_wta        adaptive-weight aggregation (seq/AdaptiveWeightAggregation.cpp:73-111)
//                   over 64-pixel x 64-disparity tiles, weights made on the fly from
//                   Lab + host tables, and the arg-min over d
#include <cuda_fp16.h>

#include "rts_common.cuh"
#include "rts_pipe.h"

namespace rts {

// ---------------------------------------------------------------------------
// cost of one (ref pixel, target pixel) pair from records

struct CostCfg {
    int k1, k2;        // RTS_COST_AD / RTS_COST_CENSUS; k2 may be RTS_COST_NONE
    int trunc1;        // truncated AD for the first cost (cross-based aggregation)
    float trunc;
    const float *lut1, *lut2;
    float l1, l2;
    int int_path;      // 1: both costs are integers < kCombineLut (integral truncation)
    int itrunc;        // integral truncation, or a large value when not truncating
};

// Integer value of one cost from records: SAD of the packed RGB bytes (the
// fourth byte is zero) or the census Hamming distance.
__device__ __forceinline__ int rec_icost(int kind, const uint4 &a, const uint4 &b, int itrunc) {
    if (kind == RTS_COST_CENSUS) return __popc(a.x ^ b.x) + __popc(a.y ^ b.y);
    return imin((int)__vsadu4(a.z, b.z), itrunc);
}

__device__ __forceinline__ float rec_cost(int kind, const uint4 &a, const uint4 &b, int use_trunc, float trunc) {
    if (kind == RTS_COST_CENSUS) {
        const uint64_t ca = ((uint64_t)a.y << 32) | a.x, cb = ((uint64_t)b.y << 32) | b.x;
        return (float)__popcll(ca ^ cb);  // seq/CensusTransform.cpp:52-60
    }
    // seq/PixelBasedCost.cpp:86-91 / :106-112 with normOrNot = 0
    const int sad = abs((int)(a.z & 0xff) - (int)(b.z & 0xff)) + abs((int)((a.z >> 8) & 0xff) - (int)((b.z >> 8) & 0xff)) +
                    abs((int)((a.z >> 16) & 0xff) - (int)((b.z >> 16) & 0xff));
    float v = (float)sad;
    if (use_trunc) v = (v > trunc) ? trunc : v;
    return v;
}

__device__ __forceinline__ float pair_cost(const uint4 &a, const uint4 &b, const CostCfg &c) {
    const float v1 = rec_cost(c.k1, a, b, c.trunc1, c.trunc);
    if (c.k2 == RTS_COST_NONE) return v1;
    const float v2 = rec_cost(c.k2, a, b, 0, 0.f);
    return __fadd_rn(combine_term(v1, c.lut1, c.l1), combine_term(v2, c.lut2, c.l2));  // seq/CombineCost.cpp:23
}

template <typename T> __device__ __forceinline__ T to_store(float v);
template <> __device__ __forceinline__ float to_store<float>(float v) { return v; }
template <> __device__ __forceinline__ __half to_store<__half>(float v) { return __float2half_rn(v); }
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__half v) { return __half2float(v); }

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
        for (int dy = -hr; dy <= hr; dy++) {
            const uint8_t *row = gray + (size_t)wrap1(y + dy, H) * W;
            for (int dx = -wr; dx <= wr; dx++, k++) code |= (uint64_t)(c > row[wrap1(x + dx, W)]) << k;
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

// ---------------------------------------------------------------------------
// Cross-based aggregation, horizontal part.  Lane = disparity.  For each x in
// order: C(x,d), P = P + C (running sum, the reference's in-place prefix,
// seq/CrossBasedAggregation.cpp:117-125).  The segment of column xs is
// P[xs+r] - P[xs-l-1] (:151-160) with l, r the min of the ref arm at xs and the
// target arm at xs-d.  Work goes in 16-column steps: 16 costs and running sums
// into registers (only the add chain is serial), then they enter a per-lane
// 64-entry ring in shared memory and the 16 segments whose right ends are now
// known are emitted.  The ring holds columns x0-48 .. x0+15, enough for
// arms <= 23.  Records are staged per warp 32 columns at a time (ref x0..x0+31,
// target x0-dbase-31 .. x0-dbase+31); the next 32 are fetched into registers
// while the current ones are consumed.
constexpr int kRing = 64;
constexpr int kHsegWarps = 2;  // keeps the static shared memory under 48 KB
constexpr int kHsegStep = 16;
constexpr int kHsegMaxArm = (kRing - kHsegStep - 1) >> 1;  // 23; also keeps l+r+1 < 64 and t, b < 32

template <typename ST, bool VOL>
__global__ void __launch_bounds__(kHsegWarps * 32) k_cross_hseg(const uint4 *__restrict__ rr, const uint4 *__restrict__ rt,
                                                               const float *__restrict__ vol, ST *__restrict__ seg,
                                                               uint16_t *__restrict__ geo, int H, int W, int D,
                                                               CostCfg cfg, int L) {
    __shared__ float pring[kHsegWarps][kRing][32];
    __shared__ uint16_t lring[kHsegWarps][kRing][32];
    __shared__ uint4 recA[kHsegWarps][32];
    __shared__ uint4 recB[kHsegWarps][64];
    __shared__ float volS[VOL ? kHsegWarps : 1][VOL ? 32 : 1][33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nch = (D + 31) >> 5;
    const int gw = blockIdx.x * kHsegWarps + warp;
    if (gw >= H * nch) return;  // only warp-level synchronisation in this kernel
    const int dbase = (gw % nch) * 32;
    const int y = gw / nch, d = dbase + lane;
    const bool active = d < D;
    const int dd = active ? d : D - 1;
    const int lo = dd - dbase;
    const size_t row = (size_t)y * W;
    float (*P)[32] = pring[warp];
    uint16_t (*LR)[32] = lring[warp];
    uint4 *RA = recA[warp], *RB = recB[warp];

    auto emit = [&](int xs) {
        const uint16_t lr = LR[xs & (kRing - 1)][lane];
        const int l = lr & 0xff, r = lr >> 8;
        int xl = xs - l - 1;
        if (xl < 0) xl = 0;  // seq/CrossBasedAggregation.cpp:153-154
        const int xr = xs + r;
        const float s = __fsub_rn(P[xr & (kRing - 1)][lane], P[xl & (kRing - 1)][lane]);
        if (active) seg[(row + xs) * D + d] = to_store<ST>(s);
    };
    auto wrapx = [&](int t) {
        t %= W;
        return t < 0 ? t + W : t;
    };
    uint4 na, nb0, nb1;
    auto fetch = [&](int x0) {
        const int t0 = x0 - dbase - 31;
        na = rr[row + imin(x0 + lane, W - 1)];
        nb0 = rt[row + wrapx(t0 + lane)];
        nb1 = rt[row + wrapx(t0 + 32 + lane)];
    };
    fetch(0);
    float acc = 0.f;
    for (int x0 = 0; x0 < W; x0 += 32) {
        __syncwarp();
        RA[lane] = na;
        RB[lane] = nb0;
        RB[lane + 32] = nb1;
        if constexpr (VOL) {
#pragma unroll 8
            for (int u = 0; u < 32; u++)
                if (x0 + u < W) volS[warp][u][lane] = vol[(row + x0 + u) * D + dd];
        }
        __syncwarp();
        if (x0 + 32 < W) fetch(x0 + 32);
#pragma unroll 1
        for (int h = 0; h < 32; h += kHsegStep) {
            const int xb = x0 + h;
            if (xb >= W) break;
            const int n = imin(kHsegStep, W - xb);
            float pv[kHsegStep];
            uint16_t lv[kHsegStep];
#pragma unroll
            for (int u = 0; u < kHsegStep; u++) {
                if (u < n) {
                    const uint4 a = RA[h + u];
                    // target column x - dd sits at index (h + u) + 31 - lo of the staged range
                    const uint4 b = RB[h + u + 31 - lo];
                    float c;
                    if constexpr (VOL) {
                        c = volS[warp][h + u][lane];
                    } else if (cfg.int_path) {
                        const int v1 = rec_icost(cfg.k1, a, b, cfg.itrunc);
                        if (cfg.k2 == RTS_COST_NONE) c = (float)v1;
                        else c = __fadd_rn(__ldg(cfg.lut1 + v1), __ldg(cfg.lut2 + rec_icost(cfg.k2, a, b, 0x7fffffff)));
                    } else {
                        c = pair_cost(a, b, cfg);
                    }
                    acc = (xb + u == 0) ? c : __fadd_rn(c, acc);  // seq/CrossBasedAggregation.cpp:123
                    pv[u] = acc;
                    const int l = imin(arm_l(a.w), arm_l(b.w)), r = imin(arm_r(a.w), arm_r(b.w));
                    lv[u] = (uint16_t)(l | (r << 8));
                    // geometry of (y, x, d): row pixel count | vertical arms (top, bottom)
                    if (active)
                        geo[(row + xb + u) * D + d] =
                            (uint16_t)((l + r + 1) | (imin(arm_t(a.w), arm_t(b.w)) << 6) | (imin(arm_b(a.w), arm_b(b.w)) << 11));
                }
            }
#pragma unroll
            for (int u = 0; u < kHsegStep; u++) {
                if (u < n) {
                    P[(xb + u) & (kRing - 1)][lane] = pv[u];
                    LR[(xb + u) & (kRing - 1)][lane] = lv[u];
                }
            }
            // columns whose right end xs + L is now in the ring
            const int xs_lo = imax(0, xb - L), xs_hi = xb + n - 1 - L;
#pragma unroll 4
            for (int xs = xs_lo; xs <= xs_hi; xs++) emit(xs);
        }
    }
    for (int xs = imax(0, W - L); xs < W; xs++) emit(xs);
}

// ---------------------------------------------------------------------------
// Cross-based aggregation, vertical part, fused with the arg-min over d.
// Block = one column x, output rows y0 .. y0+R-1 (R = 64), 8 warps.  Phase 1
// copies, for rows y0-L .. y0+R+L-1, the row segments and the geometry words
// (row pixel count | min top arm << 6 | min bottom arm << 11, written by
// k_cross_hseg) of all disparities into shared memory: 16-byte loads, all in
// flight together.  Phase 2 gives each warp whole output rows: for every
// 32-disparity chunk the lanes sum their cross rows top to bottom and divide;
// the chunk minimum comes from one redux.min over order-preserving keys plus a
// ballot (lowest lane = lowest d); chunks combine in increasing d, strict <.
constexpr int kVertThreads = 256;
constexpr int kVertRows = 64;

__device__ __forceinline__ uint32_t order_key(float v) {
    const uint32_t u = __float_as_uint(__fadd_rn(v, 0.0f));  // -0 -> +0
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

template <typename ST>
__global__ void __launch_bounds__(kVertThreads) k_cross_vert(const ST *__restrict__ seg, const uint16_t *__restrict__ geo,
                                                            uint16_t *__restrict__ raw, int *__restrict__ row_last,
                                                            int H, int W, int D, int L, int R) {
    extern __shared__ __align__(16) unsigned char vsm[];
    const int x = blockIdx.y;
    const int y0 = blockIdx.x * R, y1 = imin(H, y0 + R);
    const int ya0 = imax(0, y0 - L), ya1 = imin(H, y1 + L);
    const int nr = ya1 - ya0;
    ST *S = reinterpret_cast<ST *>(vsm);
    uint16_t *G = reinterpret_cast<uint16_t *>(vsm + (size_t)(R + 2 * L) * D * sizeof(ST));
    // phase 1: rows ya0..ya1-1 of column x are D-element runs at stride W*D
    {
        constexpr int SV = 16 / sizeof(ST);  // elements per 16-byte vector
        const int sv_row = D / SV, g_row = D / 8;
        const int ns = nr * sv_row, ng = nr * g_row;
        for (int c = threadIdx.x; c < ns + ng; c += kVertThreads) {
            if (c < ns) {
                const int ri = c / sv_row, k = c - ri * sv_row;
                reinterpret_cast<uint4 *>(S + (size_t)ri * D)[k] =
                    __ldcs(reinterpret_cast<const uint4 *>(seg + ((size_t)(ya0 + ri) * W + x) * D) + k);
            } else {
                const int c2 = c - ns;
                const int ri = c2 / g_row, k = c2 - ri * g_row;
                reinterpret_cast<uint4 *>(G + (size_t)ri * D)[k] =
                    __ldcs(reinterpret_cast<const uint4 *>(geo + ((size_t)(ya0 + ri) * W + x) * D) + k);
            }
        }
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int yo = y0 + warp; yo < y1; yo += kVertThreads / 32) {
        const int ro = yo - ya0;
        uint32_t best_key = 0xffffffffu;
        int best_d = 0;
        for (int d0 = 0; d0 < D; d0 += 32) {
            const int d = d0 + lane;
            uint32_t key = 0xffffffffu;
            if (d < D) {
                const int g = G[ro * D + d];
                const int t = (g >> 6) & 31, bo = g >> 11;
                float sum = 0.f;
                int cnt = 0;
                for (int r = ro - t; r <= ro + bo; r++) {  // seq/CrossBasedAggregation.cpp:146-164
                    sum = __fadd_rn(sum, to_f32(S[r * D + d]));
                    cnt += G[r * D + d] & 63;
                }
                key = order_key(__fdiv_rn(sum, (float)cnt));  // :166
            }
            const uint32_t m = __reduce_min_sync(0xffffffffu, key);
            if (m < best_key) {  // strict: an earlier chunk keeps ties
                const unsigned hit = __ballot_sync(0xffffffffu, key == m);
                best_key = m;
                best_d = d0 + __ffs(hit) - 1;
            }
        }
        if (lane == 0) {
            const bool found = best_d != 0;  // some d >= 1 strictly below cost[0]
            raw[(size_t)yo * W + x] = found ? (uint16_t)(0x100 | best_d) : (uint16_t)0;
            if (found) atomicMax(row_last + yo, x);
        }
    }
}

// ---------------------------------------------------------------------------
// Adaptive-weight aggregation fused with the arg-min.  Block: one row y, 64
// pixels x0..x0+63, all disparities in chunks of 64; 128 threads, each with
// 8 pixels x 4 disparities.  Warp w owns pixels 16w..16w+15 for all 64
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
constexpr int kAwTX = 64, kAwDC = 64, kAwThreads = 128;
constexpr int kAwCPitch = kAwDC + 4;
constexpr uint32_t kLabOut = 0xff000000u;  // marks a column outside the image

__global__ void k_pack_lab(const uint8_t *__restrict__ lab, uint32_t *__restrict__ out, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = (uint32_t)lab[3 * i] | ((uint32_t)lab[3 * i + 1] << 8) | ((uint32_t)lab[3 * i + 2] << 16);
}

__device__ __forceinline__ float lab_weight2(uint32_t c, uint32_t q, const float *__restrict__ G, float pwk) {
    if ((q | c) & kLabOut) return 0.f;  // tap (or padding centre) outside the image
    const uint32_t ad = __vabsdiffu4(c, q);
    return __fmul_rn(pwk, __ldg(G + __dp4a(ad, ad, 0u)));
}

template <typename CT, bool EXACT>
__global__ void __launch_bounds__(kAwThreads) k_aw_wta(const CT *__restrict__ vol, const uint32_t *__restrict__ labr,
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
    const int px0 = 16 * warp + 8 * (lane >> 4);  // pixels px0 .. px0+7 of the tile
    const int y = blockIdx.y, x0 = blockIdx.x * kAwTX;
    if (tid < kAwTX) {
        best_v[tid] = __int_as_float(0x7f800000);
        best_i[tid] = 0x7fffffff;
    }
    const bool vec = (D & 3) == 0;

    for (int dc0 = 0; dc0 < D; dc0 += kAwDC) {
        float sw[8][4], sc[8][4];
#pragma unroll
        for (int j = 0; j < 8; j++)
#pragma unroll
            for (int i = 0; i < 4; i++) sw[j][i] = sc[j][i] = 0.f;
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
            for (int kx = warp; kx < e; kx += kAwThreads / 32) {
                const float pwk = __ldg(pwrow + kx);
#pragma unroll
                for (int m = 0; m < 2; m++) wRs[kx * kAwTX + lane + 32 * m] = lab_weight2(cR[m], labRrow[lane + 32 * m + kx], G, pwk);
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    const int u = lane + 32 * m;
                    if (u < NT) {
                        uint32_t q = labTrow[u + kx];
                        if (wrapped_tile && tbase + u < 0) {
                            // the target column is t + W: its tap is column t + W + kx - r
                            const int xc = tbase + u + W + kx - r;
                            q = (xc >= 0 && xc < W) ? labt[crow + xc] : kLabOut;
                        }
                        wTs[kx * NTP + u] = lab_weight2(cT[m], q, G, pwk);
                    }
                }
            }
            __syncthreads();

            // u index of wT for (j, i): px0 + j - 4td - i + 63 = ubase + (j - i) + 3
            const int ubase = px0 - 4 * td + kAwDC - 4;
            const float *cbase = Cs + px0 * kAwCPitch + 4 * td;
            // taps in groups of 4: the 11 cost columns px0+kx0 .. px0+kx0+10 of a group
            // are loaded once and serve 8 pixels x 4 taps
#pragma unroll 1
            for (int kx0 = 0; kx0 < e; kx0 += 4) {
                const int g = imin(4, e - kx0);
                float cw[11][4];
#pragma unroll
                for (int q = 0; q < 11; q++) {
                    const float4 v = *reinterpret_cast<const float4 *>(cbase + (kx0 + q) * kAwCPitch);
                    cw[q][0] = v.x; cw[q][1] = v.y; cw[q][2] = v.z; cw[q][3] = v.w;
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    if (u < g) {
                        const int kx = kx0 + u;
                        float wr[8], wt[11];
                        const float4 a0 = *reinterpret_cast<const float4 *>(wRs + kx * kAwTX + px0);
                        const float4 a1 = *reinterpret_cast<const float4 *>(wRs + kx * kAwTX + px0 + 4);
                        wr[0] = a0.x; wr[1] = a0.y; wr[2] = a0.z; wr[3] = a0.w;
                        wr[4] = a1.x; wr[5] = a1.y; wr[6] = a1.z; wr[7] = a1.w;
                        const float4 *wp = reinterpret_cast<const float4 *>(wTs + kx * NTP + ubase);
                        const float4 b0 = wp[0], b1 = wp[1], b2 = wp[2];
                        wt[0] = b0.x; wt[1] = b0.y; wt[2] = b0.z; wt[3] = b0.w;
                        wt[4] = b1.x; wt[5] = b1.y; wt[6] = b1.z; wt[7] = b1.w;
                        wt[8] = b2.x; wt[9] = b2.y; wt[10] = b2.z;
#pragma unroll
                        for (int j = 0; j < 8; j++)
#pragma unroll
                            for (int i = 0; i < 4; i++) {
                                const float w = __fmul_rn(wr[j], wt[j - i + 3]);
                                sw[j][i] = __fadd_rn(sw[j][i], w);
                                if constexpr (EXACT) sc[j][i] = __fadd_rn(sc[j][i], __fmul_rn(cw[j + u][i], w));
                                else sc[j][i] = __fmaf_rn(cw[j + u][i], w, sc[j][i]);
                            }
                    }
                }
            }
        }
        __syncthreads();
        // score / sum of weights (seq/AdaptiveWeightAggregation.cpp:108), staged for the arg-min
        float *outs = Cs;  // [64][kAwDC + 1]
#pragma unroll
        for (int j = 0; j < 8; j++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float v = __fdiv_rn(sc[j][i], sw[j][i]);
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
// host orchestration

bool cross_fused_supported(const rts_params &p);

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
    const dim3 g((unsigned)(((long)W * D + 255) / 256), H);
    if (half) k_cost_volume<__half><<<g, 256, 0, c->stream>>>(rr, rt, (__half *)vol, H, W, D, cfg);
    else k_cost_volume<float><<<g, 256, 0, c->stream>>>(rr, rt, (float *)vol, H, W, D, cfg);
    count_launch(c);
    return check_launch(c, "cost_volume");
}

template <typename ST>
static void launch_vert(cudaStream_t s, const ST *seg, const uint16_t *geo, uint16_t *raw, int *rl, int H, int W, int D,
                        int L) {
    const int R = kVertRows;
    const size_t smem = (size_t)(R + 2 * L) * D * (sizeof(ST) + 2);
    cudaFuncSetAttribute(k_cross_vert<ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_cross_vert<ST><<<dim3((H + R - 1) / R, W), kVertThreads, smem, s>>>(seg, geo, raw, rl, H, W, D, L, R);
}

bool cross_fused_supported(const rts_params &p) {
    // 16-byte row copies in the vertical kernel need D a multiple of 8; the ring
    // of the horizontal kernel bounds the arm length
    return p.cross_arm <= kHsegMaxArm && p.disp_range % 8 == 0;
}

rts_status cross_fused(rts_ctx *c, const rts_params &p, int H, int W, const uint4 *rr, const uint4 *rt,
                       const uint32_t *ar, const uint32_t *at, const float *vol, uint16_t *raw, int *rl) {
    (void)ar;
    (void)at;
    const int D = p.disp_range, L = p.cross_arm;
    const bool half = p.precision == RTS_PREC_F16;
    CostCfg cfg;
    RTS_TRY(cost_cfg(c, p, &cfg));
    void *seg, *geo;
    const size_t ne = (size_t)H * W * D;
    RTS_TRY(scratch(c, SL_V_SEG, ne * (half ? 2 : 4), &seg));
    RTS_TRY(scratch(c, SL_V_COST2, ne * 2, &geo));
    const int nch = (D + 31) / 32;
    const unsigned blocks = (unsigned)((H * nch + kHsegWarps - 1) / kHsegWarps);
    {
        StageScope sc(c, "cross_hseg");
        auto go = [&](auto kern, auto *sp) {
            kern<<<blocks, kHsegWarps * 32, 0, c->stream>>>(rr, rt, vol, sp, (uint16_t *)geo, H, W, D, cfg, L);
        };
        if (half) {
            if (vol) go(k_cross_hseg<__half, true>, (__half *)seg);
            else go(k_cross_hseg<__half, false>, (__half *)seg);
        } else {
            if (vol) go(k_cross_hseg<float, true>, (float *)seg);
            else go(k_cross_hseg<float, false>, (float *)seg);
        }
        count_launch(c);
    }
    {
        StageScope sc(c, "cross_vert_wta");
        if (half) launch_vert<__half>(c->stream, (const __half *)seg, (const uint16_t *)geo, raw, rl, H, W, D, L);
        else launch_vert<float>(c->stream, (const float *)seg, (const uint16_t *)geo, raw, rl, H, W, D, L);
        count_launch(c);
    }
    return check_launch(c, "cross_fused");
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
    auto go = [&](auto kern, auto *v) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<grid, kAwThreads, smem, c->stream>>>(v, plr, plt, pw, g, raw, rl, cost_out, H, W, p.disp_range, e);
    };
    // plain form: bit-exact float volume; FP16 form: __half volume and fused multiply-add
    if (half) go(k_aw_wta<__half, false>, (const __half *)vol);
    else go(k_aw_wta<float, true>, (const float *)vol);
    count_launch(c);
    return check_launch(c, "aw_wta");
}

}  // namespace rts
