// rts_pipe.h -- fused per-view pipeline kernels (k_pipe.cu) used by
// rts_pipeline.cpp when the configuration has a fused path.
#pragma once

#include "rts_internal.h"

namespace rts {

// AD / census (<= 64-bit window) single or combined costs, computed on the fly
bool fast_costs(const rts_params &p);
// adaptive-weight aggregation (radius <= 16) has a fused per-view path
bool fused_supported(const rts_params &p, int H, int W);

// 16-byte per-pixel records: census code, packed RGB, packed cross arms
rts_status prep_records(rts_ctx *c, const rts_params &p, int H, int W, const uint8_t *gray, const uint8_t *rgb,
                        uint4 *rec, uint32_t *arms_out);
// cost volume [H][W][D] (float, or __half when half != 0) from records
rts_status cost_volume_fast(rts_ctx *c, const rts_params &p, int H, int W, const uint4 *rr, const uint4 *rt,
                            void *vol, int half);
// the cross-based pipeline runs over view tables (rts_views.h) when this holds
bool cross_fused_supported(const rts_params &p);
// adaptive-weight aggregation + arg-min over a float (half == 0) or __half volume
rts_status aw_fused(rts_ctx *c, const rts_params &p, int H, int W, const void *vol, int half, const uint8_t *labr,
                    const uint8_t *labt, uint16_t *raw, int *row_last, float *cost_out);

}  // namespace rts
