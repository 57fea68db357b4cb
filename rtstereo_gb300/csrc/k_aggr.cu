// k_aggr.cu -- aggregation kernels, module form (seq/ConstBlockAggregation.cpp,
// seq/CrossBasedAggregation.cpp, seq/AdaptiveWeightAggregation.cpp).
//
// These follow the reference's per-entry summation order exactly (sequential
// float adds in window order, no fused multiply-add), so their results are
// bit-identical to the reference on the same inputs.  The fused pipeline
// kernels in k_pipe.cu keep the same per-entry order with tiled data reuse.
#include "rts_common.cuh"

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
static dim3 row_grid(long per_row, int H, int threads) { return dim3((unsigned)((per_row + threads - 1) / threads), H); }

void launch_box(cudaStream_t s, const float *in, float *out, int H, int W, int D, int r) {
    k_box<<<row_grid((long)W * D, H, 256), 256, 0, s>>>(in, out, H, W, D, r);
}
void launch_find_cross(cudaStream_t s, const uint8_t *rgb, int *horz, int *vert, int H, int W, int L, int tau) {
    k_find_cross<<<row_grid(W, H, 128), 128, 0, s>>>(rgb, horz, vert, H, W, L, tau);
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
