// k_wta.cu -- winner-takes-all with the reference's carry semantics, the
// left/right cross check and small image helpers.
//
// seq/WTA.cpp:10-39 declares the winner once per call, so a pixel whose cost
// has no strictly better d >= 1 than d = 0 keeps the previous pixel's winner
// (raster order, across rows).  On the GPU this is two passes:
//   1. k_wta_local: per pixel, the first strict arg-min (arg-max) and whether
//      any d >= 1 won ("found"); found pixels raise row_last[y] to their x.
//      Warp per pixel, lane = disparity, so a warp reads its pixel's D costs
//      as whole lines; the winner is the least {wta_key, d};
//   2. k_wta_fill: one warp per row takes the incoming winner from the nearest
//      earlier row that has a found pixel, then propagates within the row with
//      a ballot scan.
// raw[p] = found ? 0x100 | winner : 0.  row_last must start at -1.
#include <algorithm>

#include "rts_common.cuh"
#include "rts_diag.cuh"

namespace rts {

constexpr int kWtaWarps = 8, kWtaPix = 4;  // warps of a block; pixels of a warp at a time
__global__ void __launch_bounds__(kWtaWarps * 32) k_wta_local(const float *__restrict__ cost, uint16_t *__restrict__ raw,
                                                              int *__restrict__ row_last, int H, int W, int D,
                                                              int argmax) {
    const int lane = threadIdx.x & 31;
    const long np = (long)H * W;
    // resident blocks stride over the pixels, a warp kWtaPix consecutive pixels at a
    // time, every pixel's loads of a 32-disparity step in flight together
    const long stride = (long)gridDim.x * kWtaWarps * kWtaPix;
    for (long p0 = ((long)blockIdx.x * kWtaWarps + (threadIdx.x >> 5)) * kWtaPix; p0 < np; p0 += stride) {
        uint32_t bk[kWtaPix], bd[kWtaPix];
#pragma unroll
        for (int j = 0; j < kWtaPix; j++) bk[j] = bd[j] = 0xffffffffu;
#pragma unroll 2
        for (int d = lane; d < D; d += 32) {
            float v[kWtaPix];
#pragma unroll
            for (int j = 0; j < kWtaPix; j++) v[j] = __ldg(cost + (p0 + j < np ? p0 + j : np - 1) * D + d);
#pragma unroll
            for (int j = 0; j < kWtaPix; j++) {
                const uint32_t k = wta_key(v[j], d, argmax);
                if (k < bk[j]) {  // a lane's d increase: a tie keeps the lower
                    bk[j] = k;
                    bd[j] = (uint32_t)d;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < kWtaPix; j++) {
            const uint32_t mn = __reduce_min_sync(0xffffffffu, bk[j]);
            const uint32_t win = __reduce_min_sync(0xffffffffu, bk[j] == mn ? bd[j] : 0xffffffffu);
            const long p = p0 + j;
            if (lane == 0 && p < np) {
                const bool found = win != 0;  // some d >= 1 strictly better than d = 0
                raw[p] = found ? (uint16_t)(0x100 | win) : (uint16_t)0;
                if (found) atomicMax(row_last + p / W, (int)(p % W));
            }
        }
    }
}

__global__ void k_wta_fill(const uint16_t *__restrict__ raw, const int *__restrict__ row_last,
                           uint8_t *__restrict__ out, int H, int W, int mirror) {
    const int lane = threadIdx.x & 31;
    const int y = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (y >= H) return;
    // incoming winner: the last found pixel of the nearest earlier row that has one
    int carry = 0;
    for (int base = y - 1; base >= 0; base -= 32) {
        const int yy = base - lane;
        const bool has = yy >= 0 && row_last[yy] >= 0;
        const unsigned m = __ballot_sync(0xffffffffu, has);
        if (m) {
            const int src = __ffs(m) - 1;  // lowest lane = highest row
            const int yy0 = base - src;
            carry = raw[(size_t)yy0 * W + row_last[yy0]] & 0xff;
            break;
        }
    }
    const uint16_t *r = raw + (size_t)y * W;
    uint8_t *o = out + (size_t)y * W;
    for (int x0 = 0; x0 < W; x0 += 32) {
        const int x = x0 + lane;
        const uint16_t v = x < W ? r[x] : (uint16_t)0;
        const unsigned fm = __ballot_sync(0xffffffffu, (v & 0x100) != 0);
        const unsigned le = fm & (0xffffffffu >> (31 - lane));
        const int src = le ? 31 - __clz(le) : 0;
        const int got = __shfl_sync(0xffffffffu, v & 0xff, src);
        const int val = le ? got : carry;
        if (x < W) o[mirror ? W - 1 - x : x] = (uint8_t)val;
        if (fm) carry = __shfl_sync(0xffffffffu, v & 0xff, 31 - __clz(fm));
    }
}

// The right view's winners from the left view's final volume (rts_diag.cuh):
// block per (row, 256 right-image pixels).
__global__ void __launch_bounds__(kDiagT) k_wta_diag(const float *__restrict__ vol, uint16_t *__restrict__ raw,
                                                     int *__restrict__ row_last, int W, int D) {
    wta_diag_item(vol, raw, row_last, W, D, blockIdx.y, blockIdx.x * kDiagT);
}

// seq/CrossCheck.cpp:10-23
__global__ void k_cross_check(const uint8_t *__restrict__ dl, const uint8_t *__restrict__ dr,
                              uint8_t *__restrict__ mask, int H, int W) {
    const int y = blockIdx.y;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    const int v = dl[(size_t)y * W + x];
    int xt = x - v;
    if (xt < 0) xt += W;        // seq/CrossCheck.cpp:16
    if (xt < 0) xt = ((xt % W) + W) % W;  // only for disparities above the width
    mask[(size_t)y * W + x] = (dr[(size_t)y * W + xt] == v) ? 1 : 0;
}

// copy with optional horizontal mirror, ch channels per pixel
__global__ void k_flip(const uint8_t *__restrict__ in, uint8_t *__restrict__ out, int H, int W, int ch, int mirror) {
    const int y = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * ch) return;
    const int x = i / ch, c = i - x * ch;
    const int xs = mirror ? W - 1 - x : x;
    out[((size_t)y * W + x) * ch + c] = in[((size_t)y * W + xs) * ch + c];
}

void launch_wta_local(cudaStream_t s, const float *cost, uint16_t *raw, int *row_last, int H, int W, int D,
                      int argmax) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 132;
    }
    const long np = (long)H * W, per_block = (long)kWtaWarps * kWtaPix;
    const long blocks = std::min((np + per_block - 1) / per_block, (long)sms * 8);
    k_wta_local<<<(unsigned)blocks, kWtaWarps * 32, 0, s>>>(cost, raw, row_last, H, W, D, argmax);
}
void launch_wta_diag(cudaStream_t s, const float *vol, uint16_t *raw, int *row_last, int H, int W, int D) {
    k_wta_diag<<<dim3((W + kDiagT - 1) / kDiagT, H), kDiagT, 0, s>>>(vol, raw, row_last, W, D);
}
void launch_wta_fill(cudaStream_t s, const uint16_t *raw, const int *row_last, uint8_t *out, int H, int W,
                     int mirror) {
    k_wta_fill<<<(H + 7) / 8, 256, 0, s>>>(raw, row_last, out, H, W, mirror);
}
void launch_cross_check(cudaStream_t s, const uint8_t *dl, const uint8_t *dr, uint8_t *mask, int H, int W) {
    k_cross_check<<<dim3((W + 127) / 128, H), 128, 0, s>>>(dl, dr, mask, H, W);
}
void launch_flip(cudaStream_t s, const uint8_t *in, uint8_t *out, int H, int W, int ch, int mirror) {
    k_flip<<<dim3((W * ch + 255) / 256, H), 256, 0, s>>>(in, out, H, W, ch, mirror);
}

}  // namespace rts

namespace rts {

// gray -> RGB by replication (what an 8-bit gray file yields when read as colour)
__global__ void k_gray_to_rgb(const uint8_t *__restrict__ g, uint8_t *__restrict__ rgb, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint8_t v = g[i];
    rgb[3 * i] = v;
    rgb[3 * i + 1] = v;
    rgb[3 * i + 2] = v;
}

void launch_gray_to_rgb(cudaStream_t s, const uint8_t *g, uint8_t *rgb, long n) {
    k_gray_to_rgb<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, rgb, n);
}

}  // namespace rts
