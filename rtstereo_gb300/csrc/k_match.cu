// k_match.cu -- matching-cost kernels (module form of seq/PixelBasedCost.cpp,
// seq/CensusTransform.cpp, seq/RankFilter.cpp, seq/ConvolveImage.cpp,
// seq/NCCDisparity.cpp, seq/CombineCost.cpp).
//
// Float arithmetic that must match the reference bit for bit is written with
// explicit round-to-nearest intrinsics in the reference's order; the library
// is compiled with -fmad=false so no multiply-add is fused behind our back.
#include "rts_common.cuh"

namespace rts {

// ---------------------------------------------------------------------------
// Absolute differences.  Grid: x-blocks over W*D of one row, y over rows; the
// cost volume is written with d fastest, so consecutive threads store
// consecutive floats.

template <typename T>
__global__ void k_ad_1ch(const T *__restrict__ ref, const T *__restrict__ tar, float *__restrict__ cost, int D,
                         int H, int W, int dir) {
    const int y = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * D) return;
    const int x = i / D, d = i - x * D;
    const int xt = tar_col(x, d, W, dir);
    const size_t row = (size_t)y * W;
    float v;
    if constexpr (sizeof(T) == 1) {
        // seq/PixelBasedCost.cpp:22 abs of an int difference
        v = (float)abs((int)ref[row + x] - (int)tar[row + xt]);
    } else {
        // seq/PixelBasedCost.cpp:48-50 float difference then sign flip
        v = __fsub_rn(ref[row + x], tar[row + xt]);
        if (v < 0) v = -v;
    }
    cost[(row + x) * D + d] = v;
}

__global__ void k_ad_color(const uint8_t *__restrict__ ref, const uint8_t *__restrict__ tar,
                           float *__restrict__ cost, int D, int H, int W, int dir, int use_trunc, float trunc,
                           int norm) {
    const int y = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * D) return;
    const int x = i / D, d = i - x * D;
    const int xt = tar_col(x, d, W, dir);
    const size_t row = (size_t)y * W;
    const uint8_t *a = ref + 3 * (row + x);
    const uint8_t *b = tar + 3 * (row + xt);
    const int sad = abs((int)a[0] - (int)b[0]) + abs((int)a[1] - (int)b[1]) + abs((int)a[2] - (int)b[2]);
    // seq/PixelBasedCost.cpp:86-91,106-112: min(sad, trunc), then (float)1/(float)3 * v
    float v = (float)sad;
    if (use_trunc) v = (v > trunc) ? trunc : v;
    if (norm) v = __fmul_rn(1.0f / 3.0f, v);
    cost[(row + x) * D + d] = v;
}

// ---------------------------------------------------------------------------
// Census.  Module form writes the reference's bool layout, one byte per bit;
// the pipeline uses packed 64-bit words (bit k of the window in word k/64).

__global__ void k_census_bits(const uint8_t *__restrict__ img, uint8_t *__restrict__ bits, int hr, int wr, int H,
                              int W) {
    const int y = blockIdx.y;
    const int bw = 2 * wr + 1, nb = (2 * hr + 1) * bw;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * nb) return;
    const int x = i / nb, k = i - x * nb;
    const int dy = k / bw - hr, dx = k - (k / bw) * bw - wr;
    const uint8_t c = img[(size_t)y * W + x];
    const uint8_t n = img[(size_t)wrap1(y + dy, H) * W + wrap1(x + dx, W)];
    bits[((size_t)y * W + x) * nb + k] = (c > n) ? 1 : 0;  // seq/CensusTransform.cpp:31 strict
}

template <int NW>
__global__ void k_census_codes(const uint8_t *__restrict__ img, uint64_t *__restrict__ codes, int hr, int wr,
                               int H, int W) {
    const int y = blockIdx.y;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    const uint8_t c = img[(size_t)y * W + x];
    uint64_t w[NW];
#pragma unroll
    for (int j = 0; j < NW; j++) w[j] = 0;
    int k = 0;
    if (NW == 1 && x >= wr && x < W - wr && y >= hr && y < H - hr) {
        // the window inside the image: no wrapping
        const uint8_t *row = img + (size_t)(y - hr) * W + x - wr;
        for (int dy = -hr; dy <= hr; dy++, row += W)
            for (int dx = 0; dx <= 2 * wr; dx++, k++) w[0] |= (uint64_t)(c > row[dx]) << k;
    } else {
        for (int dy = -hr; dy <= hr; dy++) {
            const uint8_t *row = img + (size_t)wrap1(y + dy, H) * W;
            for (int dx = -wr; dx <= wr; dx++, k++) {
                const uint64_t bit = (c > row[wrap1(x + dx, W)]) ? 1ull : 0ull;
#pragma unroll
                for (int j = 0; j < NW; j++)
                    if ((k >> 6) == j) w[j] |= bit << (k & 63);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NW; j++) codes[((size_t)y * W + x) * NW + j] = w[j];
}

template <int NW>
__global__ void k_bits_pack(const uint8_t *__restrict__ bits, uint64_t *__restrict__ codes, int nb, long npix) {
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const uint8_t *b = bits + (size_t)p * nb;
    uint64_t w[NW];
#pragma unroll
    for (int j = 0; j < NW; j++) w[j] = 0;
    for (int k = 0; k < nb; k++) {
        const uint64_t bit = b[k] ? 1ull : 0ull;
#pragma unroll
        for (int j = 0; j < NW; j++)
            if ((k >> 6) == j) w[j] |= bit << (k & 63);
    }
#pragma unroll
    for (int j = 0; j < NW; j++) codes[(size_t)p * NW + j] = w[j];
}

template <int NW>
__global__ void k_hamming(const uint64_t *__restrict__ cr, const uint64_t *__restrict__ ct, float *__restrict__ cost,
                          int D, int H, int W) {
    const int y = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * D) return;
    const int x = i / D, d = i - x * D;
    const int xt = tar_col(x, d, W, 1);
    const size_t row = (size_t)y * W;
    int cnt = 0;
#pragma unroll
    for (int j = 0; j < NW; j++) cnt += __popcll(cr[(row + x) * NW + j] ^ ct[(row + xt) * NW + j]);
    cost[(row + x) * D + d] = (float)cnt;  // seq/CensusTransform.cpp:60
}

// ---------------------------------------------------------------------------
// Rank transform (seq/RankFilter.cpp:11-35): 1 + #{q : I(q) < I(p)}, u8 wrap.
__global__ void k_rank(const uint8_t *__restrict__ img, uint8_t *__restrict__ out, int m, int H, int W) {
    const int y = blockIdx.y;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    const uint8_t c = img[(size_t)y * W + x];
    int cnt = 1;
    for (int dy = -m; dy <= m; dy++) {
        const uint8_t *row = img + (size_t)wrap1(y + dy, H) * W;
        for (int dx = -m; dx <= m; dx++) cnt += (row[wrap1(x + dx, W)] < c) ? 1 : 0;
    }
    out[(size_t)y * W + x] = (uint8_t)cnt;
}

// LoG convolution (seq/ConvolveImage.cpp:11-35): raster-order sum of rounded
// products, |.|, min 255.
__global__ void k_convolve(const uint8_t *__restrict__ img, float *__restrict__ out, const float *__restrict__ mask,
                           int H, int W, int hr, int wr) {
    const int y = blockIdx.y;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    const int mw = 2 * wr + 1;
    float acc = 0.f;
    if (x >= wr && x < W - wr && y >= hr && y < H - hr) {
        // the window inside the image: no wrapping (same products, same order)
        const uint8_t *row = img + (size_t)(y - hr) * W + x;
        for (int dy = -hr; dy <= hr; dy++, row += W) {
            const float *mk = mask + (dy + hr) * mw + wr;
            for (int dx = -wr; dx <= wr; dx++) acc = __fadd_rn(acc, __fmul_rn((float)row[dx], mk[dx]));
        }
    } else {
        for (int dy = -hr; dy <= hr; dy++) {
            const uint8_t *row = img + (size_t)wrap1(y + dy, H) * W;
            const float *mk = mask + (dy + hr) * mw + wr;
            for (int dx = -wr; dx <= wr; dx++) acc = __fadd_rn(acc, __fmul_rn((float)row[wrap1(x + dx, W)], mk[dx]));
        }
    }
    acc = (acc > 0.f) ? acc : -acc;
    out[(size_t)y * W + x] = (acc > 255.f) ? 255.f : acc;
}

// Window mean for NCC (seq/NCCDisparity.cpp:24-35): raster-order float sum / area.
// The target mean of (x, d) equals this mean at column x-d (wrapped): the same
// pixels are summed in the same order.
__global__ void k_window_mean(const uint8_t *__restrict__ img, float *__restrict__ mean, int H, int W, int hr,
                              int wr) {
    const int y = blockIdx.y;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    float s = 0.f;
    for (int dy = -hr; dy <= hr; dy++) {
        const uint8_t *row = img + (size_t)wrap1(y + dy, H) * W;
        for (int dx = -wr; dx <= wr; dx++) s = __fadd_rn(s, (float)row[wrap1(x + dx, W)]);
    }
    mean[(size_t)y * W + x] = __fdiv_rn(s, (float)((2 * hr + 1) * (2 * wr + 1)));
}

// NCC (seq/NCCDisparity.cpp:50-71): nom = sum rv*tv, den = sqrtf(sum ((rv*rv)*tv)*tv)
// in tap (raster) order, the cell written only when den != 0.  Over tiles: block per (row y, 64 pixels,
// 64 disparities), each thread 4 pixels x 4 disparities.  Per chunk of taps the
// block stages, in tap (raster) order, {rv, rv*rv} of its 64 reference pixels and
// tv of the 127 target columns t = x - d it meets (rv = I - mean, tv likewise,
// seq/NCCDisparity.cpp:55-62).  An entry's (nom, den) pair then takes per tap
//   rv*tv, ((rv*rv)*tv)*tv as scalar products, (nom, den) += (rv*tv, den term)
//   (one packed add)
// which are the reference's operations in its order.  A thread's 16 entries read
// 8 reference and 8 target floats per tap: four 16-byte shared loads, the
// target values held once (a {tv, tv} pair for a packed multiply would double
// the shared-memory traffic, which bounds the loop).
constexpr int kNccTX = 64, kNccTD = 64, kNccTaps = 49;
static_assert(sizeof(float2) * kNccTaps * kNccTX + sizeof(float) * kNccTaps * (kNccTX + kNccTD) <= kSmemOptin,
              "NCC tile exceeds the shared-memory opt-in");
// Reference rows hold float2 values in 16-byte chunks; chunk c is stored at
// c ^ ((c >> 3) & 1), so the eight 16-byte reads of a quarter warp (4 pixels
// apart) fall in distinct banks.  A quarter warp's target reads are eight
// consecutive 16-byte chunks.
__device__ __forceinline__ int ncc_swz(int u) { return (((u >> 1) ^ ((u >> 4) & 1)) << 1) | (u & 1); }

__global__ void __launch_bounds__(256) k_ncc_tiled(const uint8_t *__restrict__ ref, const uint8_t *__restrict__ tar,
                                                   const float *__restrict__ mref, const float *__restrict__ mtar,
                                                   float *__restrict__ cost, int D, int H, int W, int hr, int wr) {
    constexpr int NT = kNccTX + kNccTD - 1;       // target columns of a tile
    extern __shared__ __align__(16) unsigned char nsm[];
    float2 (*rq)[kNccTX] = reinterpret_cast<float2 (*)[kNccTX]>(nsm);                         // {rv, rv*rv}
    float (*tq)[NT + 1] = reinterpret_cast<float (*)[NT + 1]>(nsm + sizeof(float2) * kNccTaps * kNccTX);  // tv
    const int tid = threadIdx.x;
    const int px0 = 4 * (tid & 15), d0 = 4 * (tid >> 4);
    const int y = blockIdx.y, x0 = blockIdx.x * kNccTX, dc0 = blockIdx.z * kNccTD;
    const int tbase = x0 - dc0 - (kNccTD - 1);    // target column of u = 0 (before wrapping)
    const int ew = 2 * wr + 1, taps = (2 * hr + 1) * ew;
    // the tap offsets {dy, dx} of a chunk, made once per chunk
    __shared__ int2 tapoff[kNccTaps];
    float2 acc[4][4];  // (nom, den) of pixel px0 + j, disparity d0 + i
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
        for (int i = 0; i < 4; i++) acc[j][i] = make_float2(0.f, 0.f);
    for (int k0 = 0; k0 < taps; k0 += kNccTaps) {
        const int nk = min(kNccTaps, taps - k0);
        __syncthreads();  // the previous chunk is consumed
        if (tid < nk) {
            const int kk = k0 + tid, ry = kk / ew;
            tapoff[tid] = make_int2(ry - hr, kk - ry * ew - wr);
        }
        __syncthreads();
        {
            // reference cells: a thread keeps one pixel (its mean loaded once) over every
            // 4th tap of the chunk
            const int px = tid & (kNccTX - 1);
            const int x = min(x0 + px, W - 1);
            const float mr = mref[(size_t)y * W + x];
            for (int k = tid >> 6; k < nk; k += 256 / kNccTX) {
                const int2 to = tapoff[k];
                const float rv = __fsub_rn((float)ref[(size_t)wrap1(y + to.x, H) * W + wrap1(x + to.y, W)], mr);
                rq[k][ncc_swz(px)] = make_float2(rv, __fmul_rn(rv, rv));
            }
        }
        if (tid < 2 * NT) {
            // target cells: threads 0 .. 2 NT - 1 keep one column each over every other tap
            const int u = tid < NT ? tid : tid - NT;
            // t in [-W, 2W) for real entries; columns of padding entries clamped into range
            const int t = wrap1(max(min(tbase + u, W - 1), -W + 1), W);
            const float mt = mtar[(size_t)y * W + t];  // seq/NCCDisparity.cpp:37-48, same columns
            for (int k = tid < NT ? 0 : 1; k < nk; k += 2) {
                const int2 to = tapoff[k];
                const float tv = __fsub_rn((float)tar[(size_t)wrap1(y + to.x, H) * W + wrap1(t + to.y, W)], mt);
                tq[k][u] = tv;
            }
        }
        __syncthreads();
        // u index of (j, i): px0 + j - d0 - i + 63
        const int ub = px0 - d0 + kNccTD - 4;
#pragma unroll 7
        for (int k = 0; k < nk; k++) {
            float2 r[4];
            float tt[8];
            const float4 ra = *reinterpret_cast<const float4 *>(&rq[k][ncc_swz(px0)]);
            const float4 rb = *reinterpret_cast<const float4 *>(&rq[k][ncc_swz(px0 + 2)]);
            r[0] = make_float2(ra.x, ra.y); r[1] = make_float2(ra.z, ra.w);
            r[2] = make_float2(rb.x, rb.y); r[3] = make_float2(rb.z, rb.w);
            const float4 ta = *reinterpret_cast<const float4 *>(&tq[k][ub]);
            const float4 tb = *reinterpret_cast<const float4 *>(&tq[k][ub + 4]);
            tt[0] = ta.x; tt[1] = ta.y; tt[2] = ta.z; tt[3] = ta.w;
            tt[4] = tb.x; tt[5] = tb.y; tt[6] = tb.z; tt[7] = tb.w;
#pragma unroll
            for (int j = 0; j < 4; j++)
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    // scalar IEEE products (a product feeding a packed add stays unfused), the
                    // pair (rv*tv, ((rv*rv)*tv)*tv) added by one packed add
                    const float tv = tt[j - i + 3];
                    const float nt = __fmul_rn(r[j].x, tv);
                    const float dt = __fmul_rn(__fmul_rn(r[j].y, tv), tv);
                    acc[j][i] = __fadd2_rn(acc[j][i], make_float2(nt, dt));
                }
        }
    }
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int x = x0 + px0 + j, d = dc0 + d0 + i;
            if (x < W && d < D) {
                const float den = __fsqrt_rn(acc[j][i].y);  // seq/NCCDisparity.cpp:69
                if (den != 0.f) cost[((size_t)y * W + x) * D + d] = __fdiv_rn(acc[j][i].x, den);
            }
        }
}

// LoG differences combined with census Hamming distances in one pass (the
// composed k_ad_1ch<float> + k_hamming + k_combine of seq/Main.cpp:180-234 with
// LoG first and census second): the same expressions in the same order, one
// write of the volume.  A warp takes kLcPx consecutive pixels, lane = disparity.
constexpr int kLcPx = 8;

template <int NW>
__global__ void __launch_bounds__(256) k_cost_log_census(const float *__restrict__ lr, const float *__restrict__ lt,
                                                        const uint64_t *__restrict__ cr, const uint64_t *__restrict__ ct,
                                                        float *__restrict__ vol, int H, int W, int D,
                                                        const float *__restrict__ lut1, const float *__restrict__ lut2,
                                                        float lambda1, float lambda2) {
    const int y = blockIdx.y, lane = threadIdx.x & 31;
    const int xw = (blockIdx.x * 8 + (threadIdx.x >> 5)) * kLcPx;
    const size_t row = (size_t)y * W;
#pragma unroll 2
    for (int i = 0; i < kLcPx; i++) {
        const int x = xw + i;
        if (x >= W) return;
        const float a = lr[row + x];
        uint64_t ca[NW];
#pragma unroll
        for (int j = 0; j < NW; j++) ca[j] = cr[(row + x) * NW + j];
        float *out = vol + (row + x) * D;
        for (int d = lane; d < D; d += 32) {
            const int xt = x - d < 0 ? x - d + W : x - d;  // seq/PixelBasedCost.cpp:19-20
            float v1 = __fsub_rn(a, lt[row + xt]);         // seq/PixelBasedCost.cpp:48-50
            if (v1 < 0) v1 = -v1;
            int cnt = 0;
#pragma unroll
            for (int j = 0; j < NW; j++) cnt += __popcll(ca[j] ^ ct[(row + xt) * NW + j]);  // seq/CensusTransform.cpp:60
            out[d] = __fadd_rn(combine_term(v1, lut1, lambda1), combine_term((float)cnt, lut2, lambda2));
        }
    }
}

__global__ void k_combine(float *__restrict__ c1, const float *__restrict__ c2, long n, const float *__restrict__ lut1,
                          const float *__restrict__ lut2, float lambda1, float lambda2) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float a = combine_term(c1[i], lut1, lambda1);
        const float b = combine_term(c2[i], lut2, lambda2);
        c1[i] = __fadd_rn(a, b);
    }
}

// ---------------------------------------------------------------------------
// launchers

static dim3 row_grid(long per_row, int H, int threads) { return dim3((unsigned)((per_row + threads - 1) / threads), H); }

void launch_ad_gray(cudaStream_t s, const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W, int dir) {
    k_ad_1ch<uint8_t><<<row_grid((long)W * D, H, 256), 256, 0, s>>>(ref, tar, cost, D, H, W, dir);
}
void launch_ad_float(cudaStream_t s, const float *ref, const float *tar, float *cost, int D, int H, int W, int dir) {
    k_ad_1ch<float><<<row_grid((long)W * D, H, 256), 256, 0, s>>>(ref, tar, cost, D, H, W, dir);
}
void launch_ad_color(cudaStream_t s, const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W, int dir,
                     int use_trunc, float trunc, int norm) {
    k_ad_color<<<row_grid((long)W * D, H, 256), 256, 0, s>>>(ref, tar, cost, D, H, W, dir, use_trunc, trunc, norm);
}
void launch_census_bits(cudaStream_t s, const uint8_t *img, uint8_t *bits, int hr, int wr, int H, int W) {
    const long nb = (long)(2 * hr + 1) * (2 * wr + 1);
    k_census_bits<<<row_grid(W * nb, H, 256), 256, 0, s>>>(img, bits, hr, wr, H, W);
}
int census_words(int hr, int wr) {
    const int nb = (2 * hr + 1) * (2 * wr + 1);
    return nb <= 64 ? 1 : nb <= 128 ? 2 : nb <= 256 ? 4 : 0;
}
void launch_census_codes(cudaStream_t s, const uint8_t *img, uint64_t *codes, int hr, int wr, int H, int W) {
    const dim3 g = row_grid(W, H, 128);
    switch (census_words(hr, wr)) {
    case 1: k_census_codes<1><<<g, 128, 0, s>>>(img, codes, hr, wr, H, W); break;
    case 2: k_census_codes<2><<<g, 128, 0, s>>>(img, codes, hr, wr, H, W); break;
    case 4: k_census_codes<4><<<g, 128, 0, s>>>(img, codes, hr, wr, H, W); break;
    }
}
void launch_bits_pack(cudaStream_t s, const uint8_t *bits, uint64_t *codes, int nb, long npix) {
    const unsigned g = (unsigned)((npix + 127) / 128);
    if (nb <= 64) k_bits_pack<1><<<g, 128, 0, s>>>(bits, codes, nb, npix);
    else if (nb <= 128) k_bits_pack<2><<<g, 128, 0, s>>>(bits, codes, nb, npix);
    else k_bits_pack<4><<<g, 128, 0, s>>>(bits, codes, nb, npix);
}
void launch_hamming(cudaStream_t s, const uint64_t *cr, const uint64_t *ct, float *cost, int nw, int D, int H, int W) {
    const dim3 g = row_grid((long)W * D, H, 256);
    if (nw == 1) k_hamming<1><<<g, 256, 0, s>>>(cr, ct, cost, D, H, W);
    else if (nw == 2) k_hamming<2><<<g, 256, 0, s>>>(cr, ct, cost, D, H, W);
    else k_hamming<4><<<g, 256, 0, s>>>(cr, ct, cost, D, H, W);
}
void launch_rank(cudaStream_t s, const uint8_t *img, uint8_t *out, int m, int H, int W) {
    k_rank<<<row_grid(W, H, 128), 128, 0, s>>>(img, out, m, H, W);
}
void launch_convolve(cudaStream_t s, const uint8_t *img, float *out, const float *mask, int H, int W, int hr, int wr) {
    k_convolve<<<row_grid(W, H, 128), 128, 0, s>>>(img, out, mask, H, W, hr, wr);
}
void launch_window_mean(cudaStream_t s, const uint8_t *img, float *mean, int H, int W, int hr, int wr) {
    k_window_mean<<<row_grid(W, H, 128), 128, 0, s>>>(img, mean, H, W, hr, wr);
}
void launch_ncc(cudaStream_t s, const uint8_t *ref, const uint8_t *tar, const float *mref, const float *mtar,
                float *cost, int D, int H, int W, int hr, int wr) {
    const dim3 g((W + kNccTX - 1) / kNccTX, H, (D + kNccTD - 1) / kNccTD);
    const size_t smem = sizeof(float2) * kNccTaps * kNccTX + sizeof(float) * kNccTaps * (kNccTX + kNccTD);
    cudaFuncSetAttribute(k_ncc_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_ncc_tiled<<<g, 256, smem, s>>>(ref, tar, mref, mtar, cost, D, H, W, hr, wr);
}
void launch_cost_log_census(cudaStream_t s, const float *lr, const float *lt, const uint64_t *cr, const uint64_t *ct,
                            int nw, float *vol, int D, int H, int W, const float *lut1, const float *lut2,
                            float lambda1, float lambda2) {
    const dim3 g((unsigned)((W + 8 * kLcPx - 1) / (8 * kLcPx)), H);
    if (nw == 1) k_cost_log_census<1><<<g, 256, 0, s>>>(lr, lt, cr, ct, vol, H, W, D, lut1, lut2, lambda1, lambda2);
    else if (nw == 2) k_cost_log_census<2><<<g, 256, 0, s>>>(lr, lt, cr, ct, vol, H, W, D, lut1, lut2, lambda1, lambda2);
    else k_cost_log_census<4><<<g, 256, 0, s>>>(lr, lt, cr, ct, vol, H, W, D, lut1, lut2, lambda1, lambda2);
}
void launch_combine(cudaStream_t s, float *c1, const float *c2, long n, const float *lut1, const float *lut2,
                    float lambda1, float lambda2) {
    long blocks = (n + 255) / 256;
    if (blocks > 152L * 64) blocks = 152L * 64;
    k_combine<<<(unsigned)blocks, 256, 0, s>>>(c1, c2, n, lut1, lut2, lambda1, lambda2);
}

}  // namespace rts
