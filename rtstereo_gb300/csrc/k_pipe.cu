// k_pipe.cu -- fused per-view pipeline kernels.
#include "rts_common.cuh"
#include "rts_pipe.h"

namespace rts {

bool fused_supported(const rts_params &p, int H, int W) {
    (void)p;
    (void)H;
    (void)W;
    return false;
}

rts_status view_fused(rts_ctx *c, const rts_params &p, int H, int W, const uint8_t *gref, const uint8_t *gtar,
                      const uint8_t *cref, const uint8_t *ctar, const uint8_t *lref, const uint8_t *ltar,
                      uint8_t *disp, int mirror) {
    (void)p; (void)H; (void)W; (void)gref; (void)gtar; (void)cref; (void)ctar; (void)lref; (void)ltar; (void)disp;
    (void)mirror;
    return set_error(c, RTS_ERR_UNSUPPORTED, "no fused path for this configuration");
}

}  // namespace rts
