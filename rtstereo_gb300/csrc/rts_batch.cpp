// rts_batch.cpp -- batched form and serving loop (first version: pairs run
// one after another on the context stream).
#include "rts_internal.h"

using namespace rts;

extern "C" {

void rts_graph_cache_free(rts_ctx *c) { (void)c; }

rts_status rts_batch_run(rts_ctx *ctx, int n, const rts_pair *pairs, const rts_params *params, rts_out *outs) {
    if (!ctx || n < 0 || (n > 0 && (!pairs || !params || !outs))) return RTS_ERR_INVALID_ARG;
    for (int i = 0; i < n; i++) {
        rts_status s = rts_pipeline_run(ctx, RTS_DEVICE, &pairs[i], &params[i], &outs[i]);
        if (s != RTS_OK) return s;
    }
    return RTS_OK;
}

}  // extern "C"
