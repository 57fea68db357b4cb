// rts_pipe.h -- fused per-view pipeline kernels (k_pipe.cu) used by
// rts_pipeline.cpp when the configuration has a fused path.
#pragma once

#include "rts_internal.h"

namespace rts {

// True when view_fused handles this configuration (otherwise the composed
// module-kernel path runs).
bool fused_supported(const rts_params &p, int H, int W);

// One view of the pipeline with fused kernels; all pointers are device memory.
// disp receives the view's disparities, mirrored in x when `mirror` is set.
rts_status view_fused(rts_ctx *c, const rts_params &p, int H, int W, const uint8_t *gref, const uint8_t *gtar,
                      const uint8_t *cref, const uint8_t *ctar, const uint8_t *lref, const uint8_t *ltar,
                      uint8_t *disp, int mirror);

}  // namespace rts
