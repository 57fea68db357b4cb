// k_aggr.cu -- aggregation kernels, module form (seq/ConstBlockAggregation.cpp,
// seq/CrossBasedAggregation.cpp, seq/AdaptiveWeightAggregation.cpp).
//
// These follow the reference's per-entry summation order exactly (sequential
// float adds in window order, no fused multiply-add), so their results are
// bit-identical to the reference on the same inputs.  The fused pipeline
// kernels in k_pipe.cu keep the same per-entry order with tiled data reuse.
#include "rts_common.cuh"
#include "rts_tma.h"

namespace rts {

// Box mean, out of place (contract for seq/ConstBlockAggregation.cpp:11-34):
// y-outer, x-inner sequential sum over the wrapped window, / (float)area.
__global__ void k_box(const float *__restrict__ in, float *__restrict__ out, int H, int W, int D, int r) {
    const int y = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * D) return;
    const int x = i / D, d = i - x * D;
    float s = 0.f;
    for (int dy = -r; dy <= r; dy++) {
        const float *row = in + (size_t)wrap1(y + dy, H) * W * D + d;
        for (int dx = -r; dx <= r; dx++) s = __fadd_rn(s, row[(size_t)wrap1(x + dx, W) * D]);
    }
    out[((size_t)y * W + x) * D + d] = __fdiv_rn(s, (float)((2 * r + 1) * (2 * r + 1)));
}

// Box mean and arg-min in one pass (the out-of-place box of
// seq/ConstBlockAggregation.cpp:11-34 followed by seq/WTA.cpp:10-39).  Block per
// (32 x 8 pixel tile, 32 disparities): the tile and its R-pixel wrapped border
// are staged in shared memory, lane = disparity; a warp takes one row of the
// tile in groups of 8 pixels, so every staged row of 8 + 2R values feeds
// 8 x (2R + 1) adds.  Each sum is the reference's single chain, rows outer and
// columns inner.  The winner of the block's 32 disparities enters a per-pixel
// 64-bit minimum {key << 32 | d}: the key orders like the reference's strict
// comparisons (a NaN never wins, a NaN at d = 0 blocks every other d, -0 == +0).
constexpr int kBoxTX = 32, kBoxTY = 8;

template <int R, int POS>
__global__ void __launch_bounds__(256) k_box_best(const float *__restrict__ vol, unsigned long long *__restrict__ best,
                                                  int H, int W, int D, int argmax, float rcp_area) {
    constexpr int TW = kBoxTX + 2 * R, TH = kBoxTY + 2 * R, AREA = (2 * R + 1) * (2 * R + 1);
    constexpr int G = 16;  // pixels of a thread's group
    extern __shared__ float bt[];  // [TH][TW][32]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * kBoxTX, y0 = blockIdx.y * kBoxTY, d = blockIdx.z * 32 + lane;
    // the tile rows, every cell in flight at once (cp.async, zero fill past D); single
    // wrap as in seq/ConstBlockAggregation.cpp:19-24 (R < H, R < W); rows and columns
    // past the last pixel's window are never read and are clamped into range
    const bool inner = x0 >= R && x0 + kBoxTX + R <= W;
    const int dofs = d < D ? d : 0;
    const unsigned nbytes = d < D ? 4u : 0u;
    for (int i = warp; i < TH; i += 8) {
        const int yy = wrap1(imin(y0 - R + i, H - 1 + R), H);
        const float *rowp = vol + (size_t)yy * W * D + dofs;
        unsigned dst = (unsigned)__cvta_generic_to_shared(bt + i * TW * 32 + lane);
        if (inner) {
            const float *src = rowp + (size_t)(x0 - R) * D;
#pragma unroll 8
            for (int j = 0; j < TW; j++, src += D, dst += 128)
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(src), "r"(nbytes)
                             : "memory");
        } else {
            for (int j = 0; j < TW; j++, dst += 128) {
                const int xx = wrap1(imin(x0 - R + j, W - 1 + R), W);
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst),
                             "l"(rowp + (size_t)xx * D), "r"(nbytes)
                             : "memory");
            }
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    const int y = y0 + warp;
    if (y >= H) return;
#pragma unroll 1
    for (int g = 0; g < kBoxTX / G; g++) {
        // the chains of pixels (2m, 2m + 1) advance together on packed f32x2 adds
        // (each half the reference's own add, in its order)
        unsigned long long sp[G / 2];
#pragma unroll
        for (int m = 0; m < G / 2; m++) sp[m] = 0ull;
#pragma unroll
        for (int dy = 0; dy <= 2 * R; dy++) {
            constexpr int NV = G + 2 * R;  // even
            float v[NV];
            const float *rp = bt + ((warp + dy) * TW + G * g) * 32 + lane;
#pragma unroll
            for (int k = 0; k < NV; k++) v[k] = rp[k * 32];
            // {v[k], v[k + 1]} for even k (pe) and odd k (po)
            unsigned long long pe[NV / 2], po[NV / 2 - 1];
#pragma unroll
            for (int i = 0; i < NV / 2; i++) pe[i] = pack2(v[2 * i], v[2 * i + 1]);
#pragma unroll
            for (int i = 0; i < NV / 2 - 1; i++) po[i] = pack2(v[2 * i + 1], v[2 * i + 2]);
#pragma unroll
            for (int m = 0; m < G / 2; m++)
#pragma unroll
                for (int dx = 0; dx <= 2 * R; dx++) {
                    const int k = 2 * m + dx;
                    sp[m] = add2(sp[m], (k & 1) ? po[(k - 1) / 2] : pe[k / 2]);
                }
        }
        float sm[G];
#pragma unroll
        for (int j = 0; j < G; j++) sm[j] = half2_of(sp[j / 2], j & 1);
#pragma unroll
        for (int j = 0; j < G; j++) {
            const int x = x0 + G * g + j;
            float q;
            if (POS) {
                // non-negative sums of costs >= 0: the correctly rounded quotient by
                // Markstein's correction from the correctly rounded 1 / AREA
                const float q0 = __fmul_rn(sm[j], rcp_area);
                q = __fmaf_rn(__fmaf_rn(-(float)AREA, q0, sm[j]), rcp_area, q0);
            } else {
                q = __fdiv_rn(sm[j], (float)AREA);  // seq/ConstBlockAggregation.cpp:31
            }
            const uint32_t key = d < D ? wta_key(q, d, argmax) : 0xffffffffu;
            const uint32_t m = __reduce_min_sync(0xffffffffu, key);
            const uint32_t bd = __reduce_min_sync(0xffffffffu, key == m ? (uint32_t)d : 0xffffffffu);
            if (lane == 0 && x < W) atomicMin(best + (size_t)y * W + x, ((unsigned long long)m << 32) | bd);
        }
    }
}

// The same box mean and arg-min with a lane on two adjacent disparities (even D):
// block per (16 x 8 pixel tile, 64 disparities), the staged cells [TH][TW][64] so
// that a lane's pair {d, d + 1} is one 8-byte shared load that feeds a packed add
// directly (no register moves to pair pixels).  A warp takes one tile row, all 16
// pixels at once; each sum is the reference's single chain as above.
constexpr int kBoxDpTX = 16, kBoxDpTY = 8;
// the largest radius box_best_supported admits (8): staged tile + mbarrier
static_assert((size_t)(kBoxDpTX + 16) * (kBoxDpTY + 16) * 64 * sizeof(float) + 8 <= kSmemOptin,
              "box pair tile exceeds the shared-memory opt-in");
static_assert((size_t)(kBoxTX + 16) * (kBoxTY + 16) * 32 * sizeof(float) <= kSmemOptin,
              "box tile exceeds the shared-memory opt-in");

// cp.async of one tile's cells into bt2 (every cell in flight at once)
template <int R>
__device__ __forceinline__ void box_dp_stage(float2 *bt2, const float *__restrict__ vol, int H, int W, int D, int x0,
                                             int y0, int d) {
    constexpr int TW = kBoxDpTX + 2 * R, TH = kBoxDpTY + 2 * R;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // single wrap as in seq/ConstBlockAggregation.cpp:19-24; cells past the last
    // pixel's window are clamped into range (never read); zero fill past D
    const bool inner = x0 >= R && x0 + kBoxDpTX + R <= W;
    const int dofs = d < D ? d : 0;
    const unsigned nbytes = d < D ? 8u : 0u;
    for (int i = warp; i < TH; i += 8) {
        const int yy = wrap1(imin(y0 - R + i, H - 1 + R), H);
        const float *rowp = vol + (size_t)yy * W * D + dofs;
        unsigned dst = (unsigned)__cvta_generic_to_shared(bt2 + i * TW * 32 + lane);
        if (inner) {
            const float *src = rowp + (size_t)(x0 - R) * D;
#pragma unroll 8
            for (int j = 0; j < TW; j++, src += D, dst += 256)
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(nbytes)
                             : "memory");
        } else {
            for (int j = 0; j < TW; j++, dst += 256) {
                const int xx = wrap1(imin(x0 - R + j, W - 1 + R), W);
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst),
                             "l"(rowp + (size_t)xx * D), "r"(nbytes)
                             : "memory");
            }
        }
    }
}

// The sums, means and per-pixel minimum of one staged tile (warp = tile row).
// RV (the FP16 form's shared right view): also the right view's minima, for
// best_r.  The left view's entry (x, d) is the right view's (x - d mod W, d), so
// after the sums every warp stores its row's keys [16 pixels][64 disparities] in
// the staging buffer (a barrier first: the other rows' sums read it) and takes,
// for each of the 79 right pixels x0 - 64 z + k, k in [-63, 15], the minimum of
// its entries (m, m - k) in increasing disparity, entering {key, d} into best_r.
template <int R, int POS, bool RV>
__device__ __forceinline__ void box_dp_tile(float2 *bt2, unsigned long long *__restrict__ best,
                                            unsigned long long *__restrict__ best_r, int H, int W, int D, int argmax,
                                            float rcp_area, int x0, int y0, int d) {
    constexpr int TW = kBoxDpTX + 2 * R, AREA = (2 * R + 1) * (2 * R + 1);
    constexpr int G = kBoxDpTX;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int y = y0 + warp;
    const bool row_ok = y < H;
    if (!RV && !row_ok) return;
    float2 s[G];
#pragma unroll
    for (int m = 0; m < G; m++) s[m] = make_float2(0.f, 0.f);
#pragma unroll
    for (int dy = 0; dy <= 2 * R; dy++) {
        if (RV && !row_ok) break;
        const float2 *rp = bt2 + (warp + dy) * TW * 32 + lane;
        float2 v[TW];
#pragma unroll
        for (int k = 0; k < TW; k++) v[k] = rp[k * 32];
#pragma unroll
        for (int m = 0; m < G; m++)
#pragma unroll
            for (int dx = 0; dx <= 2 * R; dx++) s[m] = __fadd2_rn(s[m], v[m + dx]);
    }
    uint32_t *const kt = reinterpret_cast<uint32_t *>(bt2) + warp * (G * 64);  // RV: this row's keys
    if (RV) {
        __syncthreads();  // every row's sums are done with the staged cells
        if (!row_ok) return;
    }
    // The mean is sum / AREA correctly rounded (seq/ConstBlockAggregation.cpp:31):
    // q0 = sum * y with y = RN(1 / AREA), the residual r = sum - AREA * q0 by FMA,
    // q = RN(q0 + r * y) (Markstein's correction).  With |y - 1/AREA| <= 2^-24 / AREA
    // relative, q0 is within 1.5 ulp of the quotient, so r is an integer multiple of
    // ulp(q0) below 1.5 * AREA ulps: exact.  q0 + r * y then differs from the quotient
    // by at most 1.5 * 2^-24 ulp, less than the quotient's least distance to a
    // rounding midpoint (ulp / (2 * AREA): AREA is odd), so q is the correctly rounded
    // quotient -- for sums of either sign whose quotient is normal.  Sums of
    // non-negative costs are finite and >= +0, and their key is their bit pattern;
    // other sums outside [2^-100, 2^126] in magnitude (zero, NaN, infinity) divide.
    const uint32_t flip = argmax ? 0xffffffffu : 0u;
    const float2 ry = make_float2(rcp_area, rcp_area), na = make_float2(-(float)AREA, -(float)AREA);
#pragma unroll
    for (int m = 0; m < G; m++) {
        const int x = x0 + m;
        uint32_t k0, k1;
        if (POS) {
            const float2 q0 = __fmul2_rn(s[m], ry);
            const float2 q = __ffma2_rn(__ffma2_rn(na, q0, s[m]), ry, q0);
            k0 = (__float_as_uint(q.x) | 0x80000000u) ^ flip;  // wta_key of a float >= +0
            k1 = (__float_as_uint(q.y) | 0x80000000u) ^ flip;
        } else {
            float q[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float sm = h ? s[m].y : s[m].x, a = fabsf(sm);
                if (a >= 0x1p-100f && a <= 0x1p+126f) {
                    const float q0 = __fmul_rn(sm, rcp_area);
                    q[h] = __fmaf_rn(__fmaf_rn(-(float)AREA, q0, sm), rcp_area, q0);
                } else {
                    q[h] = __fdiv_rn(sm, (float)AREA);
                }
            }
            k0 = wta_key(q[0], d, argmax);
            k1 = wta_key(q[1], d + 1, argmax);
        }
        if (d >= D) k0 = k1 = 0xffffffffu;  // D even: d < D implies d + 1 < D
        // the lane's winner, the lower disparity on a tie
        const uint32_t key = k1 < k0 ? k1 : k0;
        const uint32_t kd = k1 < k0 ? (uint32_t)(d + 1) : (uint32_t)d;
        const uint32_t mn = __reduce_min_sync(0xffffffffu, key);
        const uint32_t bd = __reduce_min_sync(0xffffffffu, key == mn ? kd : 0xffffffffu);
        if (lane == 0 && x < W) atomicMin(best + (size_t)y * W + x, ((unsigned long long)mn << 32) | bd);
        if (RV) {
            const bool ok = x < W;  // (k0, k1 are all ones past D)
            *reinterpret_cast<uint2 *>(kt + m * 64 + 2 * lane) = make_uint2(ok ? k0 : 0xffffffffu, ok ? k1 : 0xffffffffu);
        }
    }
    if (RV) {
        __syncwarp();
        const int z64 = d - 2 * lane;  // the block's first disparity
        for (int rl = lane; rl < G + 63; rl += 32) {
            const int k = rl - 63;
            uint32_t bk = 0xffffffffu;
            int bdl = 0;
#pragma unroll
            for (int m = 0; m < G; m++) {
                const int dl = m - k;
                if (dl >= 0 && dl < 64) {
                    const uint32_t kv = kt[m * 64 + dl];
                    if (kv < bk) {  // strict: the lowest disparity keeps ties
                        bk = kv;
                        bdl = dl;
                    }
                }
            }
            if (bk != 0xffffffffu) {
                int pr = x0 - z64 + k;  // = x - d of the entries, in (-W, W)
                if (pr < 0) pr += W;
                atomicMin(best_r + (size_t)y * W + pr, ((unsigned long long)bk << 32) | (unsigned)(z64 + bdl));
            }
        }
    }
}

// Tiles whose window rows and columns all lie inside the image (no wrap) arrive
// by one TMA copy: the volume as a 3-D tensor (d, x, y) of f32, box
// (64, TW, TH) at (64 z, x0 - R, y0 - R), written densely in the [TH][TW][64]
// order the sums read, disparities past D filled with zeros; one thread issues
// it and every thread waits on an mbarrier.  The wait is bounded: a copy that has
// not landed after kTmaSpin polls counts in g_box_tma_timeouts and its block
// writes nothing.  Border tiles (wrapped cells) take the cp.async staging.
__device__ int g_box_tma_timeouts;
uint64_t box_tma_timeouts() {
    int v = 0;
    return cudaMemcpyFromSymbol(&v, g_box_tma_timeouts, sizeof(int)) == cudaSuccess ? (uint64_t)v : 0;
}

// one tile per block
template <int R, int POS, bool RV>
__global__ void __launch_bounds__(256, 2) k_box_best_dp(const __grid_constant__ CUtensorMap tmap, int use_tma,
                                                        const float *__restrict__ vol,
                                                        unsigned long long *__restrict__ best,
                                                        unsigned long long *__restrict__ best_r, int H, int W, int D,
                                                        int argmax, float rcp_area) {
    constexpr int TW = kBoxDpTX + 2 * R, TH = kBoxDpTY + 2 * R;
    constexpr uint32_t kBytes = (uint32_t)TW * TH * 64 * sizeof(float);
    // [TH][TW][32] pairs; a TMA destination must be 128-byte aligned (checked below:
    // a block whose buffer is not stages by cp.async)
    extern __shared__ __align__(128) float2 bt2[];
    __shared__ __align__(8) uint64_t bar;
    const int x0 = blockIdx.x * kBoxDpTX, y0 = blockIdx.y * kBoxDpTY, d = blockIdx.z * 64 + 2 * (threadIdx.x & 31);
    const bool tma = use_tma && x0 >= R && x0 + kBoxDpTX + R <= W && y0 >= R && y0 + kBoxDpTY + R <= H &&
                     ((uint32_t)__cvta_generic_to_shared(bt2) & 127) == 0;
    if (tma) {
        const uint32_t ba = (uint32_t)__cvta_generic_to_shared(&bar);
        if (threadIdx.x == 0) mbar_init(ba);
        __syncthreads();
        if (threadIdx.x == 0)
            tma_load_3d((uint32_t)__cvta_generic_to_shared(bt2), &tmap, (int)blockIdx.z * 64, x0 - R, y0 - R, ba,
                        kBytes);
        // the block decides together, so that no thread waits at a later barrier
        if (__syncthreads_or(!mbar_wait(ba, 0))) {
            if (threadIdx.x == 0) atomicAdd(&g_box_tma_timeouts, 1);
            mbar_wait(ba, 0);  // the copy may still land in this block's shared memory
            return;
        }
    } else {
        box_dp_stage<R>(bt2, vol, H, W, D, x0, y0, d);
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        __syncthreads();
    }
    box_dp_tile<R, POS, RV>(bt2, best, best_r, H, W, D, argmax, rcp_area, x0, y0, d);
}

// per-pixel minimum -> WTA winner word and row summary (see k_wta.cu)
// (mirror: raw and row_last in the mirrored columns of a right view)
__global__ void k_best_raw(const unsigned long long *__restrict__ best, uint16_t *__restrict__ raw,
                           int *__restrict__ row_last, int H, int W, int mirror) {
    const int y = blockIdx.y;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    const int win = (int)(best[(size_t)y * W + x] & 0xffffffffu);
    const bool found = win != 0;  // some d >= 1 strictly better than d = 0
    const int xo = mirror ? W - 1 - x : x;
    raw[(size_t)y * W + xo] = found ? (uint16_t)(0x100 | win) : (uint16_t)0;
    if (found) atomicMax(row_last + y, xo);
}

// One cross arm (seq/CrossBasedAggregation.cpp:12-100): step outward while the
// last visited pixel differs from the centre by < tau in every channel and the
// arm is shorter than L; the first failing pixel is included; stop at the edge.
__device__ __forceinline__ int cross_arm(const uint8_t *__restrict__ rgb, long centre, long step, int room, int L,
                                         int tau) {
    const int c0 = rgb[3 * centre], c1 = rgb[3 * centre + 1], c2 = rgb[3 * centre + 2];
    int len = 0, delta = 0;
    while (delta < tau && len < L && len < room) {
        len++;
        const uint8_t *q = rgb + 3 * (centre + step * len);
        delta = imax(imax(abs(c0 - (int)q[0]), abs(c1 - (int)q[1])), abs(c2 - (int)q[2]));
    }
    return len;
}

__global__ void k_find_cross(const uint8_t *__restrict__ rgb, int *__restrict__ horz, int *__restrict__ vert, int H,
                             int W, int L, int tau) {
    const int y = blockIdx.y;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    const long p = (long)y * W + x;
    vert[2 * p] = cross_arm(rgb, p, -(long)W, y, L, tau);
    vert[2 * p + 1] = cross_arm(rgb, p, (long)W, H - 1 - y, L, tau);
    horz[2 * p] = cross_arm(rgb, p, -1, x, L, tau);
    horz[2 * p + 1] = cross_arm(rgb, p, 1, W - 1 - x, L, tau);
}

// In-place running sum along x per (y, d) (seq/CrossBasedAggregation.cpp:117-125):
// one thread per chain, consecutive threads on consecutive d (coalesced).
__global__ void k_prefix_h(float *__restrict__ cost, int H, int W, int D) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)H * D) return;
    const int y = (int)(i / D), d = (int)(i - (long)y * D);
    float *p = cost + (size_t)y * W * D + d;
    float acc = p[0];
    for (int x = 1; x < W; x++) {
        acc = __fadd_rn(p[(size_t)x * D], acc);
        p[(size_t)x * D] = acc;
    }
}

// Cross-based aggregation (seq/CrossBasedAggregation.cpp:127-169).
__global__ void k_cross_aggr(const float *__restrict__ pre, float *__restrict__ out, const int *__restrict__ hr,
                             const int *__restrict__ ht, const int *__restrict__ vr, const int *__restrict__ vt, int H,
                             int W, int D) {
    const int y = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * D) return;
    const int x = i / D, d = i - x * D;
    const int xt = tar_col(x, d, W, 1);
    const long p = (long)y * W + x, q = (long)y * W + xt;
    const int t = imin(vr[2 * p], vt[2 * q]);
    const int b = imin(vr[2 * p + 1], vt[2 * q + 1]);
    float sum = 0.f;
    int cnt = 0;
    for (int yy = y - t; yy <= y + b; yy++) {
        if (yy < 0 || yy >= H) continue;
        const long pr = (long)yy * W + x, pt = (long)yy * W + xt;
        const int l = imin(hr[2 * pr], ht[2 * pt]);
        const int r = imin(hr[2 * pr + 1], ht[2 * pt + 1]);
        int xl = x - l - 1, xrr = x + r;
        if (xl < 0) xl = 0;  // :153-156 the clamped pixel is excluded from the sum, still counted
        else if (xrr >= W) xrr = W - 1;
        if (xl >= 0 && xrr < W && xl < W && xrr >= 0) {  // :157, always true for arms made by findCross
            const float *row = pre + (size_t)yy * W * D + d;
            sum = __fadd_rn(sum, __fsub_rn(row[(size_t)xrr * D], row[(size_t)xl * D]));
            cnt += r + l + 1;
        }
    }
    out[((size_t)p) * D + d] = __fdiv_rn(sum, (float)cnt);
}

// Adaptive support weights (seq/AdaptiveWeightAggregation.cpp:33-71):
// w[p][k] = pw[k] * G[|Lab(p)-Lab(q)|^2], 0 outside the image.  G is the
// host-computed expf(-sqrtf(n)/gamma_s), so the product is the reference's.
__global__ void k_compute_weights(const uint8_t *__restrict__ lab, const float *__restrict__ pw,
                                  const float *__restrict__ g, float *__restrict__ w, int H, int W, int r) {
    const int y = blockIdx.y;
    const int e = 2 * r + 1, area = e * e;
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)W * area) return;
    const int x = (int)(i / area), k = (int)(i - (long)x * area);
    const int dy = k / e - r, dx = k - (k / e) * e - r;
    const int yy = y + dy, xx = x + dx;
    float v = 0.f;
    if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
        const uint8_t *a = lab + 3 * ((size_t)y * W + x);
        const uint8_t *b = lab + 3 * ((size_t)yy * W + xx);
        const int d0 = (int)a[0] - b[0], d1 = (int)a[1] - b[1], d2 = (int)a[2] - b[2];
        v = __fmul_rn(pw[k], g[d0 * d0 + d1 * d1 + d2 * d2]);
    }
    w[((size_t)y * W + x) * area + k] = v;
}

// Adaptive-weight cost from weight arrays (seq/AdaptiveWeightAggregation.cpp:73-111):
// sequential sums over the window in raster order; weight = wR*wT, score += C*weight.
__global__ void k_aw_l2r_w(const float *__restrict__ wr, const float *__restrict__ wt, const float *__restrict__ cost,
                           float *__restrict__ out, int H, int W, int D, int r) {
    const int y = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * D) return;
    const int x = i / D, d = i - x * D;
    const int e = 2 * r + 1, area = e * e;
    const float *a = wr + ((size_t)y * W + x) * area;
    const float *b = wt + ((size_t)y * W + tar_col(x, d, W, 1)) * area;
    float sw = 0.f, sc = 0.f;
    int k = 0;
    for (int dy = -r; dy <= r; dy++) {
        const float *crow = cost + (size_t)wrap1(y + dy, H) * W * D + d;
        for (int dx = -r; dx <= r; dx++, k++) {
            const float wgt = __fmul_rn(a[k], b[k]);
            sw = __fadd_rn(sw, wgt);
            sc = __fadd_rn(sc, __fmul_rn(crow[(size_t)wrap1(x + dx, W) * D], wgt));
        }
    }
    out[((size_t)y * W + x) * D + d] = __fdiv_rn(sc, sw);
}

// R2L form, out of place (contract for seq/AdaptiveWeightAggregation.cpp:113-150):
// the weights are taken at the window pixel and at the window pixel +d.
__global__ void k_aw_r2l_w(const float *__restrict__ wr, const float *__restrict__ wt, const float *__restrict__ cost,
                           float *__restrict__ out, int H, int W, int D, int r) {
    const int y = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * D) return;
    const int x = i / D, d = i - x * D;
    const int e = 2 * r + 1, area = e * e;
    float sw = 0.f, sc = 0.f;
    int k = 0;
    for (int dy = -r; dy <= r; dy++) {
        const size_t row = (size_t)wrap1(y + dy, H) * W;
        for (int dx = -r; dx <= r; dx++, k++) {
            const int xr = wrap1(x + dx, W), xt = wrap1(x + dx + d, W);
            const float wgt = __fmul_rn(wr[(row + xr) * area + k], wt[(row + xt) * area + k]);
            sw = __fadd_rn(sw, wgt);
            sc = __fadd_rn(sc, __fmul_rn(cost[(row + xr) * D + d], wgt));
        }
    }
    out[((size_t)y * W + x) * D + d] = __fdiv_rn(sc, sw);
}

// Disparity refinement, out of place (contract for seq/CrossBasedAggregation.cpp:171-212):
// mode of the input disparities over rows y-top .. y+bottom-1 of the cross,
// segment x-left .. x+right; strict first maximum over d < D.  The histogram
// lives in shared memory, one 256-bin slice per thread.
__global__ void k_disp_refine(const uint8_t *__restrict__ in, uint8_t *__restrict__ out, const int *__restrict__ horz,
                              const int *__restrict__ vert, int H, int W, int D) {
    extern __shared__ uint16_t hist_smem[];
    uint16_t *hist = hist_smem + threadIdx.x * 256;
    const int y = blockIdx.y;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    for (int i = 0; i < 256; i++) hist[i] = 0;
    const long p = (long)y * W + x;
    const int t = vert[2 * p], b = vert[2 * p + 1];
    for (int yy = y - t; yy < y + b; yy++) {
        if (yy < 0 || yy >= H) continue;
        const long pr = (long)yy * W + x;
        int xl = x - horz[2 * pr], xr = x + horz[2 * pr + 1];
        // the reference clamps one side (:189-192); arms made by findCross never
        // reach past either edge, so clamping both only guards foreign input
        xl = imax(xl, 0);
        xr = imin(xr, W - 1);
        for (int xx = xl; xx <= xr; xx++) hist[in[(size_t)yy * W + xx]]++;
    }
    int best = hist[0], arg = 0;
    for (int i = 1; i < D; i++)
        if (hist[i] > best) {
            best = hist[i];
            arg = i;
        }
    out[p] = (uint8_t)arg;
}

// ---------------------------------------------------------------------------
// Median pre-filter of the arm images: OpenCV's medianBlur, which the OpenCL
// driver applies to both colour images before findCross
// (opencl/Main.cpp:342-343) -- per channel, the middle value of the k x k
// window, border pixels replicated.  The channels of a pixel are the bytes of
// one word.  Each byte lane's median is found bit by bit from the top: a
// candidate bit stays when at most n/2 of the n window values lie below the
// candidate, so the result is the (n/2)-th smallest value of every lane
// (counts stay below 256 for n <= 225).
constexpr int kMedTX = 32, kMedTY = 8;

template <int CH>
__global__ void __launch_bounds__(kMedTX *kMedTY)
    k_median(const uint8_t *__restrict__ in, uint8_t *__restrict__ out, int H, int W, int r) {
    extern __shared__ uint32_t mtile[];
    const int tw = kMedTX + 2 * r, th = kMedTY + 2 * r;
    const int x0 = blockIdx.x * kMedTX, y0 = blockIdx.y * kMedTY;
    for (int q = threadIdx.y * kMedTX + threadIdx.x; q < tw * th; q += kMedTX * kMedTY) {
        const int ty = q / tw, tx = q - ty * tw;
        const int yy = imin(imax(y0 - r + ty, 0), H - 1), xx = imin(imax(x0 - r + tx, 0), W - 1);
        const size_t p = (size_t)yy * W + xx;
        mtile[q] = CH == 3 ? (uint32_t)in[3 * p] | ((uint32_t)in[3 * p + 1] << 8) | ((uint32_t)in[3 * p + 2] << 16)
                           : (uint32_t)in[p];
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= W || y >= H) return;
    const int k = 2 * r + 1;
    const uint32_t half = (uint32_t)(k * k / 2) * 0x01010101u;
    uint32_t m = 0;
    for (int bit = 7; bit >= 0; bit--) {
        const uint32_t b = 0x01010101u << bit, cand = m | b;
        uint32_t cnt = 0;
        for (int dy = 0; dy < k; dy++) {
            const uint32_t *row = mtile + (threadIdx.y + dy) * tw + threadIdx.x;
            for (int dx = 0; dx < k; dx++) cnt += __vcmpltu4(row[dx], cand) & 0x01010101u;
        }
        m |= __vcmpleu4(cnt, half) & b;
    }
    const size_t p = (size_t)y * W + x;
    if (CH == 3) {
        out[3 * p] = (uint8_t)m;
        out[3 * p + 1] = (uint8_t)(m >> 8);
        out[3 * p + 2] = (uint8_t)(m >> 16);
    } else {
        out[p] = (uint8_t)m;
    }
}

// ---------------------------------------------------------------------------
static dim3 row_grid(long per_row, int H, int threads) { return dim3((unsigned)((per_row + threads - 1) / threads), H); }

void launch_box(cudaStream_t s, const float *in, float *out, int H, int W, int D, int r) {
    k_box<<<row_grid((long)W * D, H, 256), 256, 0, s>>>(in, out, H, W, D, r);
}
bool box_best_supported(int r) { return r >= 1 && r <= 8; }

bool box_best_right_supported(int r, int D) { return box_best_supported(r) && D % 2 == 0 && D > 32; }
void launch_box_best(cudaStream_t s, const float *vol, unsigned long long *best, uint16_t *raw, int *row_last, int H,
                     int W, int D, int r, int argmax, int pos, unsigned long long *best_r) {
    // disparity pairs for even D above one warp's 32; else a lane per disparity
    const bool dp = D % 2 == 0 && D > 32;
    const dim3 g = dp ? dim3((W + kBoxDpTX - 1) / kBoxDpTX, (H + kBoxDpTY - 1) / kBoxDpTY, (D + 63) / 64)
                      : dim3((W + kBoxTX - 1) / kBoxTX, (H + kBoxTY - 1) / kBoxTY, (D + 31) / 32);
    const int area = (2 * r + 1) * (2 * r + 1);
    const float rcp_area = 1.0f / (float)area;  // host IEEE division: correctly rounded
    auto go = [&](auto kern, int R) {
        const size_t smem = (size_t)(kBoxTX + 2 * R) * (kBoxTY + 2 * R) * 32 * sizeof(float);
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<g, 256, smem, s>>>(vol, best, H, W, D, argmax, rcp_area);
    };
    auto go_dp = [&](auto kern, int R) {
        const size_t smem = (size_t)(kBoxDpTX + 2 * R) * (kBoxDpTY + 2 * R) * 64 * sizeof(float);
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        CUtensorMap tm{};
        const int use_tma = volume_tensor_map(&tm, vol, H, W, D, 4, 64, kBoxDpTX + 2 * R, kBoxDpTY + 2 * R) ? 1 : 0;
        kern<<<g, 256, smem, s>>>(tm, use_tma, vol, best, best_r, H, W, D, argmax, rcp_area);
    };
#define RTS_BOX(RR)                                                \
    case RR:                                                       \
        if (dp && best_r) {                                        \
            if (pos) go_dp(k_box_best_dp<RR, 1, true>, RR);        \
            else go_dp(k_box_best_dp<RR, 0, true>, RR);            \
        } else if (dp) {                                           \
            if (pos) go_dp(k_box_best_dp<RR, 1, false>, RR);       \
            else go_dp(k_box_best_dp<RR, 0, false>, RR);           \
        } else {                                                   \
            if (pos) go(k_box_best<RR, 1>, RR);                    \
            else go(k_box_best<RR, 0>, RR);                        \
        }                                                          \
        break;
    switch (r) {
        RTS_BOX(1)
        RTS_BOX(2)
        RTS_BOX(3)
        RTS_BOX(4)
        RTS_BOX(5)
        RTS_BOX(6)
        RTS_BOX(7)
        RTS_BOX(8)
    }
#undef RTS_BOX
    k_best_raw<<<row_grid(W, H, 256), 256, 0, s>>>(best, raw, row_last, H, W, 0);
}
void launch_best_raw(cudaStream_t s, const unsigned long long *best, uint16_t *raw, int *row_last, int H, int W,
                     int mirror) {
    k_best_raw<<<row_grid(W, H, 256), 256, 0, s>>>(best, raw, row_last, H, W, mirror);
}
void launch_find_cross(cudaStream_t s, const uint8_t *rgb, int *horz, int *vert, int H, int W, int L, int tau) {
    k_find_cross<<<row_grid(W, H, 128), 128, 0, s>>>(rgb, horz, vert, H, W, L, tau);
}
void launch_median(cudaStream_t s, const uint8_t *in, uint8_t *out, int H, int W, int ch, int k) {
    const int r = k / 2;
    const dim3 g((W + kMedTX - 1) / kMedTX, (H + kMedTY - 1) / kMedTY), b(kMedTX, kMedTY);
    const size_t smem = (size_t)(kMedTX + 2 * r) * (kMedTY + 2 * r) * 4;
    if (ch == 3) k_median<3><<<g, b, smem, s>>>(in, out, H, W, r);
    else k_median<1><<<g, b, smem, s>>>(in, out, H, W, r);
}
void launch_prefix_h(cudaStream_t s, float *cost, int H, int W, int D) {
    const long n = (long)H * D;
    k_prefix_h<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(cost, H, W, D);
}
void launch_cross_aggr(cudaStream_t s, const float *pre, float *out, const int *hr, const int *ht, const int *vr,
                       const int *vt, int H, int W, int D) {
    k_cross_aggr<<<row_grid((long)W * D, H, 256), 256, 0, s>>>(pre, out, hr, ht, vr, vt, H, W, D);
}
void launch_compute_weights(cudaStream_t s, const uint8_t *lab, const float *pw, const float *g, float *w, int H, int W,
                            int r) {
    const long area = (long)(2 * r + 1) * (2 * r + 1);
    k_compute_weights<<<row_grid(W * area, H, 256), 256, 0, s>>>(lab, pw, g, w, H, W, r);
}
void launch_aw_l2r_weights(cudaStream_t s, const float *wr, const float *wt, const float *cost, float *out, int H,
                           int W, int D, int r) {
    k_aw_l2r_w<<<row_grid((long)W * D, H, 128), 128, 0, s>>>(wr, wt, cost, out, H, W, D, r);
}
void launch_aw_r2l_weights(cudaStream_t s, const float *wr, const float *wt, const float *cost, float *out, int H,
                           int W, int D, int r) {
    k_aw_r2l_w<<<row_grid((long)W * D, H, 128), 128, 0, s>>>(wr, wt, cost, out, H, W, D, r);
}
void launch_disp_refine(cudaStream_t s, const uint8_t *in, uint8_t *out, const int *horz, const int *vert, int H, int W,
                        int D) {
    const int threads = 64;
    k_disp_refine<<<row_grid(W, H, threads), threads, threads * 256 * sizeof(uint16_t), s>>>(in, out, horz, vert, H, W,
                                                                                           D);
}

}  // namespace rts
