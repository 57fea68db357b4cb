// rts_pipe.h -- fused per-view pipeline kernels (k_pipe.cu) used by
// rts_pipeline.cpp when the configuration has a fused path.
#pragma once

#include "rts_internal.h"

namespace rts {

// AD / census (<= 64-bit window) single or combined costs, computed on the fly
bool fast_costs(const rts_params &p);
// cross-based (arm <= 23) and adaptive-weight (radius <= 16) aggregation
bool fused_supported(const rts_params &p, int H, int W);

// 16-byte per-pixel records: census code, packed RGB, packed cross arms
rts_status prep_records(rts_ctx *c, const rts_params &p, int H, int W, const uint8_t *gray, const uint8_t *rgb,
                        uint4 *rec, uint32_t *arms_out);
// cost volume [H][W][D] (float, or __half when half != 0) from records
rts_status cost_volume_fast(rts_ctx *c, const rts_params &p, int H, int W, const uint4 *rr, const uint4 *rt,
                            void *vol, int half);
// cross-based aggregation + arg-min; vol == nullptr computes the cost on the fly
rts_status cross_fused(rts_ctx *c, const rts_params &p, int H, int W, const uint4 *rr, const uint4 *rt,
                       const uint32_t *ar, const uint32_t *at, const float *vol, uint16_t *raw, int *row_last);
// adaptive-weight aggregation + arg-min over a float (half == 0) or __half volume
rts_status aw_fused(rts_ctx *c, const rts_params &p, int H, int W, const void *vol, int half, const uint8_t *labr,
                    const uint8_t *labt, uint16_t *raw, int *row_last, float *cost_out);

}  // namespace rts
