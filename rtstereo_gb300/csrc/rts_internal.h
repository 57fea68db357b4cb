// rts_internal.h -- internal declarations shared by the host C++ and the CUDA
// translation units of rtstereo_gb300 (not part of the public ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rtstereo.h"

namespace rts {

// ---------------------------------------------------------------------------
// limits
constexpr int kMaxDisp = 256;      // disparities are stored in u8 (seq/WTA.cpp:12)
constexpr int kCombineLut = 1024;  // integer cost values with a host-computed 1-expf(-v/l)
constexpr int kLabDist2Max = 3 * 255 * 255;  // largest squared Lab distance (8-bit channels)

// Scratch slots of the context arena.  Each slot is a grow-only device buffer.
enum Slot {
    SL_IN0, SL_IN1, SL_IN2, SL_IN3, SL_IN4, SL_IN5,
    SL_OUT0, SL_OUT1, SL_OUT2,
    SL_TMP0, SL_TMP1, SL_TMP2, SL_TMP3,
    SL_LUT0, SL_LUT1, SL_LUTW, SL_PW, SL_RCP,
    // pipeline, per view
    SL_V_GRAY, SL_V_RGB, SL_V_LAB,          // view-ordered copies of the inputs (both images)
    SL_V_CODES, SL_V_ARMS, SL_V_AUX,        // census codes, packed arms, rank/LoG images
    SL_V_COST1, SL_V_COST2, SL_V_SEG,       // cost volumes / horizontal segment sums
    SL_V_RAW, SL_V_ROWLAST, SL_V_DISP,      // WTA winners, row summaries, view disparities
    SL_V_MEAN, SL_V_REC,                    // NCC means, fused-path pixel records
    SL_V_MED,                               // median-filtered arm images
    SL_V_FINAL,                             // the left view's final volume (FP16 form, shared right view)
    SL_BATCH0, SL_BATCH1, SL_BATCH2, SL_BATCH3,
    SL_COUNT
};

struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

struct StageTimer {
    std::string name;
    uint64_t launches = 0;
    double total_ms = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
};

struct LutKey {
    float a = -1.f, b = -1.f;
    int n = 0;
};

}  // namespace rts

struct rts_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    size_t budget = 0;
    size_t used = 0;
    std::string last_error;
    std::recursive_mutex mu;
    rts::DevBuf slots[rts::SL_COUNT];
    std::vector<rts::DevBuf> extra;  // batch / server buffers
    // cached host-computed lookup tables (the key is what the table was made for)
    rts::LutKey lut_key[2];
    bool rcp_ready = false;
    float lutw_gamma = -1.f;
    float pw_gamma = -1.f;
    int pw_rad = -1;
    std::atomic<uint64_t> launches{0};
    bool timing = false;
    std::vector<rts::StageTimer> stages;
    void *graph_cache = nullptr;  // rts::GraphCache*
    int force_tune[3] = {0, 0, 0};  // cross-based views: {vert_rows, grid_mult, persistent}; vert_rows 0: autotune
};

namespace rts {

// error helpers -------------------------------------------------------------
rts_status set_error(rts_ctx *c, rts_status s, const std::string &msg);
rts_status cuda_check(rts_ctx *c, cudaError_t e, const char *what);
#define RTS_CU(ctx, call)                                             \
    do {                                                              \
        cudaError_t _e = (call);                                      \
        if (_e != cudaSuccess) return ::rts::cuda_check(ctx, _e, #call); \
    } while (0)
#define RTS_TRY(expr)                      \
    do {                                   \
        rts_status _s = (expr);            \
        if (_s != RTS_OK) return _s;       \
    } while (0)

// arena ----------------------------------------------------------------------
// Returns a device buffer of at least `bytes` for `slot` (grown if needed).
rts_status scratch(rts_ctx *c, int slot, size_t bytes, void **out);
rts_status dev_alloc(rts_ctx *c, size_t bytes, void **out);
void dev_free(rts_ctx *c, void *p, size_t bytes);

// host <-> device staging for RTS_HOST calls -------------------------------
// Input: returns a device pointer holding `bytes` from `src` (copied if HOST).
rts_status stage_in(rts_ctx *c, rts_mem m, int slot, const void *src, size_t bytes, const void **dev);
// Output: returns a device pointer to write to (slot scratch if HOST).
rts_status stage_out(rts_ctx *c, rts_mem m, int slot, void *dst, size_t bytes, void **dev);
// In/out buffer: copies in (HOST) and returns a device pointer.
rts_status stage_inout(rts_ctx *c, rts_mem m, int slot, void *buf, size_t bytes, void **dev);
// Copies a staged output back to the host and synchronises (HOST only).
rts_status finish_out(rts_ctx *c, rts_mem m, void *dst, const void *dev, size_t bytes);
rts_status finish(rts_ctx *c, rts_mem m);

// launch bookkeeping (kernel counter, stage timing) ------------------------
void count_launch(rts_ctx *c, int n = 1);
struct StageScope {
    rts_ctx *c;
    int idx;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    StageScope(rts_ctx *c, const char *name);
    ~StageScope();
};
rts_status check_launch(rts_ctx *c, const char *what);
// Opts `kern` into `smem` bytes of dynamic shared memory, checking the result
// (a request above the device's opt-in limit fails here, with the kernel's name,
// rather than later as a generic launch error).
template <typename K> rts_status set_smem(rts_ctx *c, K kern, size_t smem, const char *what) {
    int dev = 0, limit = 0;
    RTS_CU(c, cudaGetDevice(&dev));
    RTS_CU(c, cudaDeviceGetAttribute(&limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (smem > (size_t)limit)
        return set_error(c, RTS_ERR_UNSUPPORTED, std::string(what) + ": " + std::to_string(smem) +
                                                     " bytes of shared memory exceed the device's " +
                                                     std::to_string(limit));
    return cuda_check(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), what);
}

// host-computed tables (glibc expf/sqrtf, same as the reference) ----------
// combine LUT: T[v] = 1 - expf(-(float)v / lambda), v in [0, kCombineLut)
rts_status combine_luts(rts_ctx *c, float lambda1, float lambda2, const float **l1, const float **l2);
// correctly rounded reciprocals R[n] = 1 / (float)n, n in [1, kRecipMax]
constexpr int kRecipMax = 47 * 47;  // largest cross of arm 23: (2 * 23 + 1)^2 pixels
rts_status recip_table(rts_ctx *c, const float **r);
// Lab weight LUT: G[n] = expf(-sqrtf((float)n) / gamma_s), n in [0, kLabDist2Max]
rts_status lab_weight_lut(rts_ctx *c, float gamma_s, const float **g);
// proximity weights pw[k] (seq/AdaptiveWeightAggregation.cpp:11-18), device copy
rts_status prox_weights(rts_ctx *c, float gamma_p, int rad, const float **pw);
void host_prox_weight(float *pw, float gamma_p, int rad);

// ---------------------------------------------------------------------------
// kernel launchers (defined in the .cu files); all enqueue on `s`.
// k_match.cu
void launch_ad_gray(cudaStream_t s, const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W, int dir);
void launch_ad_float(cudaStream_t s, const float *ref, const float *tar, float *cost, int D, int H, int W, int dir);
void launch_ad_color(cudaStream_t s, const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W,
                     int dir, int use_trunc, float trunc, int norm);
void launch_census_bits(cudaStream_t s, const uint8_t *img, uint8_t *bits, int hr, int wr, int H, int W);
int census_words(int hr, int wr);
void launch_census_codes(cudaStream_t s, const uint8_t *img, uint64_t *codes, int hr, int wr, int H, int W);
void launch_bits_pack(cudaStream_t s, const uint8_t *bits, uint64_t *codes, int nb, long npix);
void launch_hamming(cudaStream_t s, const uint64_t *cr, const uint64_t *ct, float *cost, int nw, int D, int H,
                    int W);
void launch_rank(cudaStream_t s, const uint8_t *img, uint8_t *out, int m, int H, int W);
void launch_convolve(cudaStream_t s, const uint8_t *img, float *out, const float *mask, int H, int W, int hr,
                     int wr);
void launch_window_mean(cudaStream_t s, const uint8_t *img, float *mean, int H, int W, int hr, int wr);
void launch_ncc(cudaStream_t s, const uint8_t *ref, const uint8_t *tar, const float *mref, const float *mtar,
                float *cost, int D, int H, int W, int hr, int wr);
// LoG first cost combined with census second cost in one pass (nw census words)
void launch_cost_log_census(cudaStream_t s, const float *lr, const float *lt, const uint64_t *cr, const uint64_t *ct,
                            int nw, float *vol, int D, int H, int W, const float *lut1, const float *lut2,
                            float lambda1, float lambda2);
void launch_combine(cudaStream_t s, float *c1, const float *c2, long n, const float *lut1, const float *lut2,
                    float lambda1, float lambda2);
// TMA copies whose bounded wait gave up (device counters of k_aggr.cu / k_pipe.cu)
uint64_t box_tma_timeouts();
uint64_t aw_tma_timeouts();
// k_aggr.cu
void launch_box(cudaStream_t s, const float *in, float *out, int H, int W, int D, int r);
// box mean + WTA winners in one pass (radius 1..8): best[] must hold all ones;
// writes raw / row_last as launch_wta_local does (two launches); pos: every cost
// is >= 0 (the fast exact division applies)
bool box_best_supported(int r);
void launch_box_best(cudaStream_t s, const float *vol, unsigned long long *best, uint16_t *raw, int *row_last, int H,
                     int W, int D, int r, int argmax, int pos, unsigned long long *best_r = nullptr);
// launch_box_best can also enter the right view's minima {key, d} (the left
// view's entries (x, d) at right pixel x - d mod W) into best_r (all ones at the
// start): the disparity-pair kernel only (even D above 32)
bool box_best_right_supported(int r, int D);
// best [H][W] minima -> raw / row_last (launch_wta_local's), mirrored columns if asked
void launch_best_raw(cudaStream_t s, const unsigned long long *best, uint16_t *raw, int *row_last, int H, int W,
                     int mirror);
void launch_find_cross(cudaStream_t s, const uint8_t *rgb, int *horz, int *vert, int H, int W, int L, int tau);
// per-channel median of the k x k window, borders replicated (ch 1 or 3)
inline bool median_ksize_ok(int k) { return k >= 3 && k <= 15 && (k & 1); }
void launch_median(cudaStream_t s, const uint8_t *in, uint8_t *out, int H, int W, int ch, int k);
void launch_prefix_h(cudaStream_t s, float *cost, int H, int W, int D);
void launch_cross_aggr(cudaStream_t s, const float *pre, float *out, const int *hr, const int *ht, const int *vr,
                       const int *vt, int H, int W, int D);
void launch_compute_weights(cudaStream_t s, const uint8_t *lab, const float *pw, const float *g, float *w, int H,
                            int W, int r);
void launch_aw_l2r_weights(cudaStream_t s, const float *wr, const float *wt, const float *cost, float *out, int H,
                           int W, int D, int r);
void launch_aw_r2l_weights(cudaStream_t s, const float *wr, const float *wt, const float *cost, float *out, int H,
                           int W, int D, int r);
void launch_disp_refine(cudaStream_t s, const uint8_t *in, uint8_t *out, const int *horz, const int *vert, int H,
                        int W, int D);
// k_wta.cu
void launch_wta_local(cudaStream_t s, const float *cost, uint16_t *raw, int *row_last, int H, int W, int D,
                      int argmax);
void launch_wta_fill(cudaStream_t s, const uint16_t *raw, const int *row_last, uint8_t *out, int H, int W,
                     int mirror);
// the right view's winners from the left view's final volume [H][W][D] (its
// diagonals (x + d mod W, d)); raw / row_last in the right view's mirrored columns
void launch_wta_diag(cudaStream_t s, const float *vol, uint16_t *raw, int *row_last, int H, int W, int D);
void launch_cross_check(cudaStream_t s, const uint8_t *dl, const uint8_t *dr, uint8_t *mask, int H, int W);
void launch_flip(cudaStream_t s, const uint8_t *in, uint8_t *out, int H, int W, int ch, int mirror);
void launch_gray_to_rgb(cudaStream_t s, const uint8_t *g, uint8_t *rgb, long n);

}  // namespace rts
