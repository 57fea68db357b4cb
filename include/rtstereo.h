/*
 * rtstereo.h -- C ABI of rtstereo_gb300, a GB300 (sm_103a) implementation of
 * the per-frame local stereo-matching pipeline of rtstereo (seq/).
 *
 * Drop-in boundary.  The reference's module API is the set of free C++
 * functions in the seq headers (caller-owned buffers, void return, no error report).
 * Each rts_<name> below replaces the seq function of the same name, takes the
 * same arguments in the same order and meaning, and adds
 *   - an rts_ctx* (device, stream, scratch arena, HBM budget) and
 *   - an rts_mem flag saying whether the pointers are HOST or DEVICE memory,
 * and returns an rts_status instead of void.  With RTS_HOST the call copies the
 * inputs to the device, runs, copies the outputs back and synchronises; with
 * RTS_DEVICE it only enqueues work on the context's stream.
 * include/rts_seq_compat.hpp re-exposes the exact seq signatures on top.
 *
 * Layouts are the reference's: gray u8 [H][W]; RGB/Lab u8 [H][W][3];
 * cost volume f32 [H][W][D] (cost[d + D*(x + W*y)]); census bits u8 0/1
 * [H][W][(2h+1)(2w+1)]; arms int32 [H][W][2].  rdim = H rows, cdim = W columns.
 */
#ifndef RTSTEREO_H
#define RTSTEREO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rts_status {
    RTS_OK = 0,
    RTS_ERR_INVALID_ARG = 1, /* bad size, null pointer, unsupported parameter */
    RTS_ERR_OOM = 2,         /* device allocation failed or HBM budget exceeded */
    RTS_ERR_CUDA = 3,        /* a CUDA call failed; see rts_ctx_last_error */
    RTS_ERR_TIMEOUT = 4,     /* a bounded wait gave up */
    RTS_ERR_UNSUPPORTED = 5, /* no CUDA device / extension not usable here */
    RTS_ERR_BUSY = 6,        /* admission refused: no slot or no memory free */
    RTS_ERR_CANCELLED = 7    /* a serving request was cancelled */
} rts_status;

typedef enum rts_mem { RTS_HOST = 0, RTS_DEVICE = 1 } rts_mem;

typedef struct rts_ctx rts_ctx;

/* ---- context ----------------------------------------------------------- */
/* hbm_budget: bytes of device memory the context may hold (0 = no limit). */
rts_status rts_ctx_create(rts_ctx **out, int device, size_t hbm_budget);
void rts_ctx_destroy(rts_ctx *ctx);
/* Run on an external stream (a cudaStream_t); NULL restores the own stream. */
rts_status rts_ctx_set_stream(rts_ctx *ctx, void *cuda_stream);
void *rts_ctx_stream(rts_ctx *ctx);
rts_status rts_ctx_synchronize(rts_ctx *ctx);
size_t rts_ctx_bytes_in_use(const rts_ctx *ctx);
const char *rts_ctx_last_error(const rts_ctx *ctx);
const char *rts_status_string(rts_status s);
/* Number of kernels this library has launched since the context was created. */
uint64_t rts_ctx_kernel_launches(const rts_ctx *ctx);
/* Fixes the tile of the cross-based view kernels instead of the autotuner's
 * choice: rows per vertical-aggregation item (a strip of one column), persistent
 * row-segment blocks per SM, and persistent (1) or one block per item (0);
 * vert_rows 0 restores the autotuner.  For tests and tuning: every tile gives the
 * same results. */
rts_status rts_ctx_force_cross_tune(rts_ctx *ctx, int vert_rows, int grid_mult, int persistent);
/* Tile copies (TMA) on the context's device whose bounded completion wait gave up
 * since the library was loaded; their blocks wrote no result.  0 in normal use. */
uint64_t rts_ctx_tma_timeouts(const rts_ctx *ctx);
/* Per-stage timing with CUDA events on the context stream (tracing). */
rts_status rts_ctx_enable_stage_timing(rts_ctx *ctx, int enable);
/* Copies up to max stage records (name, launches, total ms) accumulated since the
 * last reset; returns the number of stages. */
int rts_ctx_stage_times(rts_ctx *ctx, const char **names, uint64_t *launches, double *total_ms, int max);
void rts_ctx_reset_stage_times(rts_ctx *ctx);

/* ---- matching cost: seq/PixelBasedCost.h:6-13 -------------------------- */
/* seq/PixelBasedCost.cpp:13-24 */
rts_status rts_pixelBasedL2R(rts_ctx *, rts_mem, const uint8_t *ref_image, const uint8_t *tar_image,
                             float *cost, int dispRange, int rdim, int cdim);
/* seq/PixelBasedCost.cpp:26-37 */
rts_status rts_pixelBasedR2L(rts_ctx *, rts_mem, const uint8_t *ref_image, const uint8_t *tar_image,
                             float *cost, int dispRange, int rdim, int cdim);
/* seq/PixelBasedCost.cpp:39-53 */
rts_status rts_pixelBasedCostL2R_Float(rts_ctx *, rts_mem, const float *ref_image, const float *tar_image,
                                       float *cost, int dispRange, int rdim, int cdim);
/* seq/PixelBasedCost.cpp:55-69 */
rts_status rts_pixelBasedCostR2L_Float(rts_ctx *, rts_mem, const float *ref_image, const float *tar_image,
                                       float *cost, int dispRange, int rdim, int cdim);
/* seq/PixelBasedCost.cpp:72-92 (overload without truncation) */
rts_status rts_pixelBasedCostL2R_Color(rts_ctx *, rts_mem, const uint8_t *ref_image, const uint8_t *tar_image,
                                       float *cost, int dispRange, int rdim, int cdim, int normOrNot);
/* seq/PixelBasedCost.cpp:94-114 (overload with float trunc) */
rts_status rts_pixelBasedCostL2R_Color_trunc(rts_ctx *, rts_mem, const uint8_t *ref_image,
                                             const uint8_t *tar_image, float *cost, int dispRange, int rdim,
                                             int cdim, float trunc, int normOrNot);
/* seq/PixelBasedCost.cpp:116-136 (declared as pixelBasedCostR2L_Color in seq/PixelBasedCost.h:11) */
rts_status rts_pixelBasedR2L_Color(rts_ctx *, rts_mem, const uint8_t *ref_image, const uint8_t *tar_image,
                                   float *cost, int dispRange, int rdim, int cdim, int normOrNot);
/* seq/PixelBasedCost.cpp:138-158 */
rts_status rts_pixelBasedR2L_Color_trunc(rts_ctx *, rts_mem, const uint8_t *ref_image, const uint8_t *tar_image,
                                         float *cost, int dispRange, int rdim, int cdim, float trunc,
                                         int normOrNot);

/* ---- census: seq/CensusTransform.h:1-2 ----------------------------------- */
/* seq/CensusTransform.cpp:11-37; censusTrans is bool/u8 [H][W][(2h+1)(2w+1)] */
rts_status rts_calcCensusTrans(rts_ctx *, rts_mem, const uint8_t *img, uint8_t *censusTrans, int maskHrad,
                               int maskWrad, int rdim, int cdim);
/* seq/CensusTransform.cpp:39-62 */
rts_status rts_calcHammingDist(rts_ctx *, rts_mem, const uint8_t *censusTrnsRef, const uint8_t *censusTrnsTar,
                               float *cost, int maskHrad, int maskWrad, int rdim, int cdim, int dispRange);

/* ---- rank / LoG / NCC / combine ----------------------------------------- */
/* seq/RankFilter.cpp:11-35 (maskSize is a radius) */
rts_status rts_calculateRankFilt(rts_ctx *, rts_mem, const uint8_t *img, uint8_t *outImg, int maskSize, int rdim,
                                 int cdim);
/* seq/ConvolveImage.cpp:11-35; mask is a host or device array like the images */
rts_status rts_convolveImage(rts_ctx *, rts_mem, const uint8_t *img, float *outIm, const float *mask, int rdim,
                             int cdim, int maskHrad, int maskWrad);
/* seq/NCCDisparity.cpp:11-73; cells with a zero denominator are left unwritten */
rts_status rts_calcNCCDispL2R(rts_ctx *, rts_mem, const uint8_t *ref_image, const uint8_t *tar_image, float *cost,
                              int dispRange, int rdim, int cdim, int maskHrad, int maskWrad);
/* seq/CombineCost.cpp:11-25, in place into cost1 */
rts_status rts_combineCost(rts_ctx *, rts_mem, float *cost1, const float *cost2, float lambda1, float lambda2,
                           int rdim, int cdim, int dispRange);

/* ---- aggregation ----------------------------------------------------------- */
/* seq/ConstBlockAggregation.cpp:11-34.  In place into cost, with the window
 * read from the unmodified input (the reference reads already-averaged
 * neighbours; that serial recurrence is not reproduced). */
rts_status rts_boxAggregate(rts_ctx *, rts_mem, float *cost, int rdim, int cdim, int dispRange, int wndwRad);
/* seq/CrossBasedAggregation.cpp:102-115 (arm length 17, threshold 20) */
rts_status rts_findCross(rts_ctx *, rts_mem, const uint8_t *image, int *HorzOffset, int *VertOffset, int rdim,
                         int cdim);
/* same with explicit arm length and colour threshold (seq/CrossBasedAggregation.h:8-9) */
rts_status rts_findCross_ex(rts_ctx *, rts_mem, const uint8_t *image, int *HorzOffset, int *VertOffset, int rdim,
                            int cdim, int arm_len, int tau);
/* seq/CrossBasedAggregation.cpp:117-125, in place */
rts_status rts_aggregate_cost_horizontal(rts_ctx *, rts_mem, float *cost_image, int rdim, int cdim, int dispRange);
/* seq/CrossBasedAggregation.cpp:127-169 */
rts_status rts_cross_stereo_aggregation(rts_ctx *, rts_mem, const float *cost_image, float *cost_new_image,
                                        const int *HorzOffset_ref, const int *HorzOffset_tar,
                                        const int *VertOffset_ref, const int *VertOffset_tar, int rdim, int cdim,
                                        int dispRange);
/* seq/CrossBasedAggregation.cpp:171-212.  In place, with the votes taken from
 * the unmodified input disparities. */
rts_status rts_disp_refinement(rts_ctx *, rts_mem, uint8_t *dispIm, const int *HorzOffset, const int *VertOffset,
                               int rdim, int cdim, int dispRange);
/* Median pre-filter of the cross-arm images, in place: per channel the median
 * of the maskSize x maskSize window (odd, 3..15), border pixels replicated --
 * the OpenCV medianBlur(img, img, 3) the OpenCL driver applies to both colour
 * images before findCross (opencl/Main.cpp:342-343).  seq declares
 * medianFilt(image, maskSize) without sizes and never defines it
 * (seq/CrossBasedAggregation.h:12); channels is 1 or 3 (interleaved). */
rts_status rts_medianFilt(rts_ctx *, rts_mem, uint8_t *image, int rdim, int cdim, int channels, int maskSize);
/* seq/AdaptiveWeightAggregation.cpp:11-18 (host arithmetic; proxWeight follows mem) */
rts_status rts_calcProxWeight(rts_ctx *, rts_mem, float *proxWeight, float gamma_proximity, int maskRad);
/* seq/AdaptiveWeightAggregation.cpp:33-71; weights f32 [H][W][(2r+1)^2] */
rts_status rts_computeWeights(rts_ctx *, rts_mem, float *weights, const float *proxWeight, const uint8_t *LABImage,
                              float gamma_similarity, int rdim, int cdim, int maskRad);
/* seq/AdaptiveWeightAggregation.cpp:73-111 */
rts_status rts_calcAWCostL2R(rts_ctx *, rts_mem, const float *weightRef, const float *weightTar, const float *cost,
                             float *newCost, int rdim, int cdim, int dispRange, int maskRad);
/* seq/AdaptiveWeightAggregation.cpp:113-150.  In place, with the window read
 * from the unmodified input. */
rts_status rts_calcAWCostR2L(rts_ctx *, rts_mem, const float *weightRef, const float *weightTar, float *cost,
                             int rdim, int cdim, int dispRange, int maskRad);

/* ---- disparity ------------------------------------------------------------ */
/* seq/WTA.cpp:10-24 (including the carry of the previous pixel's winner) */
rts_status rts_WTA(rts_ctx *, rts_mem, const float *cost, uint8_t *winners, int rdim, int cdim, int dispRange);
/* seq/WTA.cpp:26-39 */
rts_status rts_WTA_NCC(rts_ctx *, rts_mem, const float *cost, uint8_t *winners, int rdim, int cdim, int dispRange);
/* No counterpart in the reference.  rts_WTA for callers that cannot allocate
 * device memory (a host that fixes its device memory at start-up, or a frame
 * loop that must not hit the device-wide synchronisation of cudaMalloc/cudaFree).
 * DEVICE pointers only, enqueued on cuda_stream (NULL: the legacy default
 * stream); no context.  Its scratch is a static device array built into the
 * library (about 4 MiB, held by every GPU that loads the library until exit):
 * rdim*cdim <= 2,097,152 and rdim <= 8192, else RTS_ERR_INVALID_ARG.  The first
 * call on a device looks up that array's device address with the device current,
 * so make it before any stream capture.  All calls share the array: calls whose
 * work overlaps on the GPU race and must be serialised by the caller. */
rts_status rts_WTA_noalloc(const float *cost, uint8_t *winners, int rdim, int cdim, int dispRange, void *cuda_stream);
/* seq/CrossCheck.cpp:10-23 */
rts_status rts_cross_check(rts_ctx *, rts_mem, const uint8_t *ref_disparity, const uint8_t *tar_disparity,
                           uint8_t *cross_check_image, int rdim, int cdim);

/* ---- whole pipeline: seq/Main.cpp:180-257 ------------------------------- */
enum { RTS_COST_NONE = 0, RTS_COST_AD = 1, RTS_COST_RANK = 2, RTS_COST_CENSUS = 3, RTS_COST_LOG = 4,
       RTS_COST_NCC = 5 };
enum { RTS_AGGR_NONE = 0, RTS_AGGR_BOX = 1, RTS_AGGR_AW = 2, RTS_AGGR_CROSS = 3 };
enum { RTS_PREC_F32 = 0, RTS_PREC_F16 = 1 };

typedef struct rts_params {
    int cost1;        /* seq argv[4]: 1 AD, 2 rank, 3 census, 4 LoG; 5 NCC (single cost) */
    int cost2;        /* seq argv[5]: 0 single cost, else a second cost combined by combineCost */
    int aggr;         /* seq argv[6]: 0 none, 1 box, 2 adaptive weight, 3 cross-based */
    float lambda1;    /* seq argv[8] */
    float lambda2;    /* seq argv[9] */
    int disp_range;   /* seq argv[3], 1..256 and <= width */
    int census_hrad, census_wrad; /* seq/Main.cpp:107-108: 4, 3 */
    int rank_rad;     /* seq/Main.cpp:111: 7 */
    int ncc_hrad, ncc_wrad;       /* seq/Main.cpp:119-120: 1, 1 */
    int box_rad;      /* seq/Main.cpp:102: 1 */
    int aw_rad;       /* seq/Main.cpp:122: 16 */
    float aw_gamma_s; /* seq/Main.cpp:123: 7 */
    float aw_gamma_p; /* seq/Main.cpp:124: 36 */
    int cross_arm;    /* seq/CrossBasedAggregation.h:8: 17 */
    int cross_tau;    /* seq/CrossBasedAggregation.h:9: 20 */
    float ad_trunc;   /* seq/Main.cpp:128: 24 (AD first cost with cross-based aggregation) */
    int right_view;   /* 1: right view as flip(L2R(flip R, flip L)) and the cross-check mask */
    int precision;    /* RTS_PREC_F32 (plain) or RTS_PREC_F16 (fp16 storage, fp32 accumulation; with
                         adaptive weights the right view is read from the left view's final volume,
                         equal to the mirrored pipeline's up to the order of its sums) */
    int median_ksize; /* 0: off; odd 3..15 (cross-based only): the arms are found on median-filtered
                         copies of the colour images, the costs on the unfiltered ones, as the OpenCL
                         driver does (opencl/Main.cpp:342-343, medianBlur with 3) */
} rts_params;

void rts_params_default(rts_params *p);

typedef struct rts_pair {
    int width, height;
    const uint8_t *left_gray, *right_gray; /* [H][W] */
    const uint8_t *left_rgb, *right_rgb;   /* [H][W][3]; NULL: the gray image replicated */
    const uint8_t *left_lab, *right_lab;   /* [H][W][3]; required for adaptive weights */
} rts_pair;

typedef struct rts_out {
    uint8_t *disp_left;  /* [H][W] */
    uint8_t *disp_right; /* [H][W] (right_view) or NULL */
    uint8_t *mask;       /* [H][W] cross-check 0/1 (right_view) or NULL */
    float *cost_left;    /* optional [H][W][D] final left cost volume or NULL (the plain form, or the
                            FP16 form with adaptive weights of radius <= 16 or with box aggregation) */
} rts_out;

rts_status rts_pipeline_run(rts_ctx *, rts_mem, const rts_pair *pair, const rts_params *params, rts_out *out);

/* ---- batched form ---------------------------------------------------------- */
/* n pairs of any sizes and disparity ranges; DEVICE buffers; one launch per
 * stage over a work list of (pair, tile), replayed from a CUDA graph cached per
 * batch shape. */
rts_status rts_batch_run(rts_ctx *, int n, const rts_pair *pairs, const rts_params *params, rts_out *outs);

/* ---- serving loop (continuous batching) -------------------------------------- */
/* Requests (HOST buffers, copied on submit) are admitted in arrival order while
 * a slot and enough of the server's device pool are free, launched as batches
 * on a ring of streams (a batch overlaps with the ones still running) and
 * completed by polling.  All requests of a server share every parameter except
 * disp_range; the pipeline is the fused cross-based one. */
typedef struct rts_server rts_server;
typedef struct rts_server_config {
    size_t hbm_budget;   /* bytes of cost-volume memory admitted at once (e.g. 40 GB) */
    int max_inflight;    /* slots: pairs on the device at once */
    int max_batch;       /* pairs launched together */
    int precision;       /* RTS_PREC_F32 or RTS_PREC_F16 */
    long long priority_pixels; /* 0: one class; else requests of at least this many pixels
                                  run alone on high-priority streams (older first), the others
                                  in batches that do not start while such a request runs
                                  (unless the oldest has waited 8 ms) */
} rts_server_config;

typedef struct rts_request_stats {
    double submit_ms, start_ms, done_ms; /* host clock, ms since server creation */
} rts_request_stats;

rts_status rts_server_create(rts_server **out, rts_ctx *ctx, const rts_server_config *cfg);
void rts_server_destroy(rts_server *s);
/* Copies the HOST inputs (pair) on submit; outputs land in HOST out buffers
 * (pinned ones are written by the device directly, pageable ones through the
 * server's pinned staging; a cancelled request that is already running may
 * still write pinned outputs). */
rts_status rts_server_submit(rts_server *s, const rts_pair *pair, const rts_params *params, rts_out *out,
                             uint64_t *ticket);
/* 1 done, 0 pending, <0 an error status (negated) */
int rts_server_poll(rts_server *s, uint64_t ticket);
rts_status rts_server_wait(rts_server *s, uint64_t ticket, double timeout_ms, rts_request_stats *stats);
/* A pending request is dropped at once; a running one when its batch leaves
 * the device.  wait / poll then report RTS_ERR_CANCELLED for the ticket (for the
 * 4096 most recently cancelled tickets). */
rts_status rts_server_cancel(rts_server *s, uint64_t ticket);
/* Requests the server still holds: pending, running, or finished and not yet
 * collected by rts_server_wait (cancelled ones are not held). */
long rts_server_tracked(rts_server *s);
/* Drives admission and completion; call from the submitting thread or let
 * rts_server_wait drive it. */
rts_status rts_server_progress(rts_server *s);

/* ---- synthetic random-dot stereo pairs (host) ------------------------------ */
/* Left: uniform u8 texture smoothed by a 3x3 box ((sum+4)/9, clamp-to-edge).
 * Right(y,x) = Left(y, clamp(x + d(y,x))) + N(0, sigma), rounded half away and
 * clipped; d: background bg_disp, n_rects random rectangles with d in
 * [0, max_disp), n_planes slanted planes.  gt_disp may be NULL. */
rts_status rts_synth_pair(uint64_t seed, int width, int height, int max_disp, int n_rects, int n_planes,
                          float sigma, int bg_disp, uint8_t *left_gray, uint8_t *right_gray, uint8_t *gt_disp);
/* gray -> RGB by replication */
void rts_gray_to_rgb(const uint8_t *gray, uint8_t *rgb, int width, int height);
/* RGB -> 8-bit CIE L*a*b* (sRGB, D65; L*255/100, a+128, b+128) */
void rts_rgb_to_lab(const uint8_t *rgb, uint8_t *lab, int width, int height);

#ifdef __cplusplus
}
#endif
#endif
