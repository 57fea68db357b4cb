// rts_diag.cuh -- the right view's local arg-min read from the left view's final
// volume (the FP16 form: adaptive weights, and a box whose volume is returned;
// otherwise the box + arg-min kernel forms the same minima itself).
//
// In exact arithmetic the right view's final cost of (pixel x, disparity d) --
// the mirrored left-to-right pipeline's -- equals the left view's at
// ((x + d) mod W, d).  Adaptive weights: both are sums over the same taps of the
// same terms, the product of the same two pixels' weights (zero where either
// window leaves the image, seq/AdaptiveWeightAggregation.cpp:47-55) times the
// same symmetric matching cost (AD and census distances do not depend on which
// image is the reference).  Box: both windows wrap at the image edges
// (seq/ConstBlockAggregation.cpp:19-24), so they hold the same costs.  The right
// view adds them in mirrored tap order.  The FP16 form uses this identity; its
// sums may then round differently from the mirrored pipeline's, so the plain
// form does not.  (The cross-based sums do not share it:
// seq/CrossBasedAggregation.cpp:152-153 drops the first cost of a row segment
// that starts at column 0 of the view, a different column in the mirrored view.)
#pragma once

#include "rts_common.cuh"

namespace rts {

constexpr int kDiagT = 256;       // threads of a block = right-image pixels of an item
constexpr int kDiagRows = kDiagT + 31;  // left pixels staged per 32-disparity chunk

// One item: row y, right-image pixels x0 .. x0 + kDiagT - 1.  Per 32-disparity
// chunk c the block stages the left pixels (x0 + 32c + i) mod W, i < kDiagRows,
// with their 32 costs (row pitch 33, so that thread t's reads at (t + j, j) fall
// in distinct banks; every load of a warp in flight before its stores), then
// thread t scans its diagonal.  The scan is the reference's WTA
// (seq/WTA.cpp:10-24: the first strict minimum, "found" when some d >= 1 beats
// d = 0); raw and row_last are in the right view's (mirrored) columns.
__device__ __forceinline__ void wta_diag_item(const float *__restrict__ vol, uint16_t *__restrict__ raw,
                                              int *__restrict__ row_last, int W, int D, int y, int x0) {
    __shared__ float st[kDiagRows * 33];
    constexpr int NI = (kDiagRows + kDiagT / 32 - 1) / (kDiagT / 32);  // staged rows per warp
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int x = x0 + t;
    const float *row = vol + (size_t)y * W * D;
    float best = 0.f;
    int win = 0;
    bool found = false;
    // the staged cells of chunk c, loaded into registers one chunk ahead so that
    // the next chunk's reads are in flight while this one is scanned
    float v[NI];
    auto load = [&](int c) {
        const int d = 32 * c + lane;
        // column of staged row i = warp + 8k: one modulo per chunk, then steps of 8
        // wrapped by a subtraction (W >= 8), or by the modulo for narrower images
        int col = (x0 + 32 * c + warp) % W;
#pragma unroll
        for (int k = 0; k < NI; k++) {
            const int i = warp + (kDiagT / 32) * k;
            v[k] = 0.f;
            if (i < kDiagRows && d < D) v[k] = row[(size_t)col * D + d];
            col += kDiagT / 32;
            col = col >= W ? (W >= kDiagT / 32 ? col - W : col % W) : col;
        }
    };
    load(0);
    for (int c = 0; 32 * c < D; c++) {
        __syncthreads();  // the previous chunk's readers are done
#pragma unroll
        for (int k = 0; k < NI; k++) {
            const int i = warp + (kDiagT / 32) * k;
            if (i < kDiagRows) st[i * 33 + lane] = v[k];
        }
        __syncthreads();
        if (32 * (c + 1) < D) load(c + 1);
        if (x < W) {
            const int jn = imin(32, D - 32 * c);
            for (int j = 0; j < jn; j++) {
                const float u = st[(t + j) * 33 + j];
                if (c == 0 && j == 0) {
                    best = u;
                } else if (u < best) {
                    best = u;
                    win = 32 * c + j;
                    found = true;
                }
            }
        }
    }
    if (x < W) {
        const int xm = W - 1 - x;
        raw[(size_t)y * W + xm] = found ? (uint16_t)(0x100 | win) : (uint16_t)0;
        if (found) atomicMax(row_last + y, xm);
    }
}

}  // namespace rts
