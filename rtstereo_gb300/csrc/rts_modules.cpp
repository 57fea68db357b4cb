// rts_modules.cpp -- the C-ABI module entry points: one rts_<name> per
// function of the reference's seq/ module API (seq/*.h), same arguments, plus
// a context and a HOST/DEVICE memory flag.  Each validates its sizes (the
// reference checks nothing; out-of-range sizes are reported here instead of
// reading out of bounds), stages HOST buffers through the context arena,
// launches the kernels on the context stream and, for HOST calls, copies the
// results back and synchronises.
#include <string.h>

#include <vector>

#include "rts_internal.h"

using namespace rts;

namespace {

struct Call {
    rts_ctx *c;
    std::unique_lock<std::recursive_mutex> lock;
    rts_status st = RTS_OK;
    explicit Call(rts_ctx *ctx) : c(ctx) {
        if (!c) {
            st = RTS_ERR_INVALID_ARG;
            return;
        }
        lock = std::unique_lock<std::recursive_mutex>(c->mu);
        if (cudaSetDevice(c->device) != cudaSuccess) st = set_error(c, RTS_ERR_CUDA, "cudaSetDevice failed");
    }
};

rts_status bad(rts_ctx *c, const char *msg) { return set_error(c, RTS_ERR_INVALID_ARG, msg); }

// dims common to the cost-volume functions: 1 <= D <= 256, D <= W (single wrap)
rts_status check_dims(rts_ctx *c, int D, int H, int W) {
    if (H <= 0 || W <= 0) return bad(c, "rdim and cdim must be positive");
    if (D <= 0 || D > kMaxDisp) return bad(c, "dispRange must be in 1..256");
    if (D > W) return bad(c, "dispRange must not exceed cdim (the target column wraps once)");
    if ((size_t)W * (size_t)D >= (1u << 31)) return bad(c, "cdim*dispRange too large");
    return RTS_OK;
}

rts_status check_img(rts_ctx *c, int H, int W) {
    if (H <= 0 || W <= 0) return bad(c, "rdim and cdim must be positive");
    if ((size_t)W * 3 * 256 >= (1u << 31)) return bad(c, "cdim too large");
    return RTS_OK;
}

#define PROLOGUE(ctx)              \
    Call call_(ctx);               \
    if (call_.st != RTS_OK) return call_.st; \
    rts_ctx *c = call_.c;          \
    (void)c

size_t vol(int D, int H, int W) { return (size_t)D * H * W * sizeof(float); }
size_t pix(int H, int W) { return (size_t)H * W; }

rts_status ad_color(rts_ctx *c, rts_mem m, const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W,
                    int dir, int use_trunc, float trunc, int norm) {
    RTS_TRY(check_dims(c, D, H, W));
    const void *dr, *dt;
    void *dc;
    RTS_TRY(stage_in(c, m, SL_IN0, ref, pix(H, W) * 3, &dr));
    RTS_TRY(stage_in(c, m, SL_IN1, tar, pix(H, W) * 3, &dt));
    RTS_TRY(stage_out(c, m, SL_OUT0, cost, vol(D, H, W), &dc));
    {
        StageScope sc(c, "ad_color");
        launch_ad_color(c->stream, (const uint8_t *)dr, (const uint8_t *)dt, (float *)dc, D, H, W, dir, use_trunc,
                        trunc, norm);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "ad_color"));
    RTS_TRY(finish_out(c, m, cost, dc, vol(D, H, W)));
    return finish(c, m);
}

rts_status ad_gray(rts_ctx *c, rts_mem m, const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W,
                   int dir) {
    RTS_TRY(check_dims(c, D, H, W));
    const void *dr, *dt;
    void *dc;
    RTS_TRY(stage_in(c, m, SL_IN0, ref, pix(H, W), &dr));
    RTS_TRY(stage_in(c, m, SL_IN1, tar, pix(H, W), &dt));
    RTS_TRY(stage_out(c, m, SL_OUT0, cost, vol(D, H, W), &dc));
    {
        StageScope sc(c, "ad_gray");
        launch_ad_gray(c->stream, (const uint8_t *)dr, (const uint8_t *)dt, (float *)dc, D, H, W, dir);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "ad_gray"));
    RTS_TRY(finish_out(c, m, cost, dc, vol(D, H, W)));
    return finish(c, m);
}

rts_status ad_float(rts_ctx *c, rts_mem m, const float *ref, const float *tar, float *cost, int D, int H, int W,
                    int dir) {
    RTS_TRY(check_dims(c, D, H, W));
    const void *dr, *dt;
    void *dc;
    RTS_TRY(stage_in(c, m, SL_IN0, ref, pix(H, W) * 4, &dr));
    RTS_TRY(stage_in(c, m, SL_IN1, tar, pix(H, W) * 4, &dt));
    RTS_TRY(stage_out(c, m, SL_OUT0, cost, vol(D, H, W), &dc));
    {
        StageScope sc(c, "ad_float");
        launch_ad_float(c->stream, (const float *)dr, (const float *)dt, (float *)dc, D, H, W, dir);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "ad_float"));
    RTS_TRY(finish_out(c, m, cost, dc, vol(D, H, W)));
    return finish(c, m);
}

rts_status wta(rts_ctx *c, rts_mem m, const float *cost, uint8_t *win, int H, int W, int D, int argmax) {
    RTS_TRY(check_dims(c, D, H, W));
    const void *dc;
    void *dw, *raw, *rl;
    RTS_TRY(stage_in(c, m, SL_IN0, cost, vol(D, H, W), &dc));
    RTS_TRY(stage_out(c, m, SL_OUT0, win, pix(H, W), &dw));
    RTS_TRY(scratch(c, SL_TMP0, pix(H, W) * 2, &raw));
    RTS_TRY(scratch(c, SL_TMP1, (size_t)H * 4, &rl));
    {
        StageScope sc(c, "wta");
        RTS_CU(c, cudaMemsetAsync(rl, 0xff, (size_t)H * 4, c->stream));
        launch_wta_local(c->stream, (const float *)dc, (uint16_t *)raw, (int *)rl, H, W, D, argmax);
        launch_wta_fill(c->stream, (const uint16_t *)raw, (const int *)rl, (uint8_t *)dw, H, W, 0);
        count_launch(c, 2);
    }
    RTS_TRY(check_launch(c, "wta"));
    RTS_TRY(finish_out(c, m, win, dw, pix(H, W)));
    return finish(c, m);
}

}  // namespace

extern "C" {

// ---- matching cost ---------------------------------------------------------

rts_status rts_pixelBasedL2R(rts_ctx *ctx, rts_mem m, const uint8_t *ref, const uint8_t *tar, float *cost, int D,
                             int H, int W) {
    PROLOGUE(ctx);
    return ad_gray(c, m, ref, tar, cost, D, H, W, 1);
}

rts_status rts_pixelBasedR2L(rts_ctx *ctx, rts_mem m, const uint8_t *ref, const uint8_t *tar, float *cost, int D,
                             int H, int W) {
    PROLOGUE(ctx);
    return ad_gray(c, m, ref, tar, cost, D, H, W, -1);
}

rts_status rts_pixelBasedCostL2R_Float(rts_ctx *ctx, rts_mem m, const float *ref, const float *tar, float *cost, int D,
                                       int H, int W) {
    PROLOGUE(ctx);
    return ad_float(c, m, ref, tar, cost, D, H, W, 1);
}

rts_status rts_pixelBasedCostR2L_Float(rts_ctx *ctx, rts_mem m, const float *ref, const float *tar, float *cost, int D,
                                       int H, int W) {
    PROLOGUE(ctx);
    return ad_float(c, m, ref, tar, cost, D, H, W, -1);
}

rts_status rts_pixelBasedCostL2R_Color(rts_ctx *ctx, rts_mem m, const uint8_t *ref, const uint8_t *tar, float *cost,
                                       int D, int H, int W, int norm) {
    PROLOGUE(ctx);
    return ad_color(c, m, ref, tar, cost, D, H, W, 1, 0, 0.f, norm);
}

rts_status rts_pixelBasedCostL2R_Color_trunc(rts_ctx *ctx, rts_mem m, const uint8_t *ref, const uint8_t *tar,
                                             float *cost, int D, int H, int W, float trunc, int norm) {
    PROLOGUE(ctx);
    return ad_color(c, m, ref, tar, cost, D, H, W, 1, 1, trunc, norm);
}

rts_status rts_pixelBasedR2L_Color(rts_ctx *ctx, rts_mem m, const uint8_t *ref, const uint8_t *tar, float *cost, int D,
                                   int H, int W, int norm) {
    PROLOGUE(ctx);
    return ad_color(c, m, ref, tar, cost, D, H, W, -1, 0, 0.f, norm);
}

rts_status rts_pixelBasedR2L_Color_trunc(rts_ctx *ctx, rts_mem m, const uint8_t *ref, const uint8_t *tar, float *cost,
                                         int D, int H, int W, float trunc, int norm) {
    PROLOGUE(ctx);
    return ad_color(c, m, ref, tar, cost, D, H, W, -1, 1, trunc, norm);
}

// ---- census ----------------------------------------------------------------

rts_status rts_calcCensusTrans(rts_ctx *ctx, rts_mem m, const uint8_t *img, uint8_t *bits, int hr, int wr, int H,
                               int W) {
    PROLOGUE(ctx);
    RTS_TRY(check_img(c, H, W));
    if (hr < 0 || wr < 0 || hr >= H || wr >= W) return bad(c, "census radii must be >= 0 and smaller than the image");
    const size_t nb = (size_t)(2 * hr + 1) * (2 * wr + 1);
    if ((size_t)W * nb >= (1u << 31)) return bad(c, "census window too large for this width");
    const void *di;
    void *db;
    RTS_TRY(stage_in(c, m, SL_IN0, img, pix(H, W), &di));
    RTS_TRY(stage_out(c, m, SL_OUT0, bits, pix(H, W) * nb, &db));
    {
        StageScope sc(c, "census_bits");
        launch_census_bits(c->stream, (const uint8_t *)di, (uint8_t *)db, hr, wr, H, W);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "census_bits"));
    RTS_TRY(finish_out(c, m, bits, db, pix(H, W) * nb));
    return finish(c, m);
}

rts_status rts_calcHammingDist(rts_ctx *ctx, rts_mem m, const uint8_t *bref, const uint8_t *btar, float *cost, int hr,
                               int wr, int H, int W, int D) {
    PROLOGUE(ctx);
    RTS_TRY(check_dims(c, D, H, W));
    if (hr < 0 || wr < 0) return bad(c, "census radii must be >= 0");
    const int nb = (2 * hr + 1) * (2 * wr + 1);
    const int nw = census_words(hr, wr);
    if (nw == 0) return bad(c, "census windows above 256 bits are not supported");
    const void *da, *dbb;
    void *dc, *ca, *cb;
    RTS_TRY(stage_in(c, m, SL_IN0, bref, pix(H, W) * nb, &da));
    RTS_TRY(stage_in(c, m, SL_IN1, btar, pix(H, W) * nb, &dbb));
    RTS_TRY(stage_out(c, m, SL_OUT0, cost, vol(D, H, W), &dc));
    RTS_TRY(scratch(c, SL_TMP0, pix(H, W) * nw * 8, &ca));
    RTS_TRY(scratch(c, SL_TMP1, pix(H, W) * nw * 8, &cb));
    {
        StageScope sc(c, "hamming");
        launch_bits_pack(c->stream, (const uint8_t *)da, (uint64_t *)ca, nb, (long)pix(H, W));
        launch_bits_pack(c->stream, (const uint8_t *)dbb, (uint64_t *)cb, nb, (long)pix(H, W));
        launch_hamming(c->stream, (const uint64_t *)ca, (const uint64_t *)cb, (float *)dc, nw, D, H, W);
        count_launch(c, 3);
    }
    RTS_TRY(check_launch(c, "hamming"));
    RTS_TRY(finish_out(c, m, cost, dc, vol(D, H, W)));
    return finish(c, m);
}

// ---- rank / LoG / NCC / combine -------------------------------------------

rts_status rts_calculateRankFilt(rts_ctx *ctx, rts_mem m, const uint8_t *img, uint8_t *out, int ms, int H, int W) {
    PROLOGUE(ctx);
    RTS_TRY(check_img(c, H, W));
    if (ms < 0 || ms >= H || ms >= W) return bad(c, "rank radius must be >= 0 and smaller than the image");
    const void *di;
    void *dout;
    RTS_TRY(stage_in(c, m, SL_IN0, img, pix(H, W), &di));
    RTS_TRY(stage_out(c, m, SL_OUT0, out, pix(H, W), &dout));
    {
        StageScope sc(c, "rank");
        launch_rank(c->stream, (const uint8_t *)di, (uint8_t *)dout, ms, H, W);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "rank"));
    RTS_TRY(finish_out(c, m, out, dout, pix(H, W)));
    return finish(c, m);
}

rts_status rts_convolveImage(rts_ctx *ctx, rts_mem m, const uint8_t *img, float *out, const float *mask, int H, int W,
                             int hr, int wr) {
    PROLOGUE(ctx);
    RTS_TRY(check_img(c, H, W));
    if (hr < 0 || wr < 0 || hr >= H || wr >= W) return bad(c, "mask radii must be >= 0 and smaller than the image");
    const void *di, *dm;
    void *dout;
    RTS_TRY(stage_in(c, m, SL_IN0, img, pix(H, W), &di));
    RTS_TRY(stage_in(c, m, SL_IN1, mask, (size_t)(2 * hr + 1) * (2 * wr + 1) * 4, &dm));
    RTS_TRY(stage_out(c, m, SL_OUT0, out, pix(H, W) * 4, &dout));
    {
        StageScope sc(c, "convolve");
        launch_convolve(c->stream, (const uint8_t *)di, (float *)dout, (const float *)dm, H, W, hr, wr);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "convolve"));
    RTS_TRY(finish_out(c, m, out, dout, pix(H, W) * 4));
    return finish(c, m);
}

rts_status rts_calcNCCDispL2R(rts_ctx *ctx, rts_mem m, const uint8_t *ref, const uint8_t *tar, float *cost, int D,
                              int H, int W, int hr, int wr) {
    PROLOGUE(ctx);
    RTS_TRY(check_dims(c, D, H, W));
    if (hr < 0 || wr < 0 || hr >= H || wr + D > W) return bad(c, "NCC window radii out of range for this image");
    const void *dr, *dt;
    void *dc, *mr, *mt;
    RTS_TRY(stage_in(c, m, SL_IN0, ref, pix(H, W), &dr));
    RTS_TRY(stage_in(c, m, SL_IN1, tar, pix(H, W), &dt));
    // unwritten cells keep the caller's values: stage the output in/out
    RTS_TRY(stage_inout(c, m, SL_OUT0, cost, vol(D, H, W), &dc));
    RTS_TRY(scratch(c, SL_TMP0, pix(H, W) * 4, &mr));
    RTS_TRY(scratch(c, SL_TMP1, pix(H, W) * 4, &mt));
    {
        StageScope sc(c, "ncc");
        launch_window_mean(c->stream, (const uint8_t *)dr, (float *)mr, H, W, hr, wr);
        launch_window_mean(c->stream, (const uint8_t *)dt, (float *)mt, H, W, hr, wr);
        launch_ncc(c->stream, (const uint8_t *)dr, (const uint8_t *)dt, (const float *)mr, (const float *)mt,
                   (float *)dc, D, H, W, hr, wr);
        count_launch(c, 3);
    }
    RTS_TRY(check_launch(c, "ncc"));
    RTS_TRY(finish_out(c, m, cost, dc, vol(D, H, W)));
    return finish(c, m);
}

rts_status rts_combineCost(rts_ctx *ctx, rts_mem m, float *c1, const float *c2, float l1, float l2, int H, int W,
                           int D) {
    PROLOGUE(ctx);
    if (H <= 0 || W <= 0 || D <= 0) return bad(c, "sizes must be positive");
    const float *lut1, *lut2;
    RTS_TRY(combine_luts(c, l1, l2, &lut1, &lut2));
    void *d1;
    const void *d2;
    RTS_TRY(stage_inout(c, m, SL_IN0, c1, vol(D, H, W), &d1));
    RTS_TRY(stage_in(c, m, SL_IN1, c2, vol(D, H, W), &d2));
    {
        StageScope sc(c, "combine");
        launch_combine(c->stream, (float *)d1, (const float *)d2, (long)D * H * W, lut1, lut2, l1, l2);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "combine"));
    RTS_TRY(finish_out(c, m, c1, d1, vol(D, H, W)));
    return finish(c, m);
}

// ---- aggregation -------------------------------------------------------------

rts_status rts_boxAggregate(rts_ctx *ctx, rts_mem m, float *cost, int H, int W, int D, int r) {
    PROLOGUE(ctx);
    if (H <= 0 || W <= 0 || D <= 0 || D > kMaxDisp) return bad(c, "bad sizes");
    if (r < 0 || r >= H || r >= W) return bad(c, "window radius must be >= 0 and smaller than the image");
    void *dc, *tmp;
    RTS_TRY(stage_inout(c, m, SL_IN0, cost, vol(D, H, W), &dc));
    RTS_TRY(scratch(c, SL_TMP0, vol(D, H, W), &tmp));
    {
        StageScope sc(c, "box");
        launch_box(c->stream, (const float *)dc, (float *)tmp, H, W, D, r);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "box"));
    if (m == RTS_DEVICE) {
        RTS_CU(c, cudaMemcpyAsync(cost, tmp, vol(D, H, W), cudaMemcpyDeviceToDevice, c->stream));
        return RTS_OK;
    }
    RTS_TRY(finish_out(c, m, cost, tmp, vol(D, H, W)));
    return finish(c, m);
}

rts_status rts_findCross_ex(rts_ctx *ctx, rts_mem m, const uint8_t *rgb, int *horz, int *vert, int H, int W, int L,
                            int tau) {
    PROLOGUE(ctx);
    RTS_TRY(check_img(c, H, W));
    if (L < 0 || L > 255) return bad(c, "arm length must be in 0..255");
    const void *di;
    void *dh, *dv;
    RTS_TRY(stage_in(c, m, SL_IN0, rgb, pix(H, W) * 3, &di));
    RTS_TRY(stage_out(c, m, SL_OUT0, horz, pix(H, W) * 8, &dh));
    RTS_TRY(stage_out(c, m, SL_OUT1, vert, pix(H, W) * 8, &dv));
    {
        StageScope sc(c, "find_cross");
        launch_find_cross(c->stream, (const uint8_t *)di, (int *)dh, (int *)dv, H, W, L, tau);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "find_cross"));
    RTS_TRY(finish_out(c, m, horz, dh, pix(H, W) * 8));
    RTS_TRY(finish_out(c, m, vert, dv, pix(H, W) * 8));
    return finish(c, m);
}

rts_status rts_findCross(rts_ctx *ctx, rts_mem m, const uint8_t *rgb, int *horz, int *vert, int H, int W) {
    return rts_findCross_ex(ctx, m, rgb, horz, vert, H, W, 17, 20);
}

rts_status rts_aggregate_cost_horizontal(rts_ctx *ctx, rts_mem m, float *cost, int H, int W, int D) {
    PROLOGUE(ctx);
    if (H <= 0 || W <= 0 || D <= 0) return bad(c, "sizes must be positive");
    void *dc;
    RTS_TRY(stage_inout(c, m, SL_IN0, cost, vol(D, H, W), &dc));
    {
        StageScope sc(c, "prefix_h");
        launch_prefix_h(c->stream, (float *)dc, H, W, D);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "prefix_h"));
    RTS_TRY(finish_out(c, m, cost, dc, vol(D, H, W)));
    return finish(c, m);
}

rts_status rts_cross_stereo_aggregation(rts_ctx *ctx, rts_mem m, const float *pre, float *out, const int *hr,
                                        const int *ht, const int *vr, const int *vt, int H, int W, int D) {
    PROLOGUE(ctx);
    RTS_TRY(check_dims(c, D, H, W));
    const void *dp, *a, *b, *cc, *dd;
    void *dout;
    RTS_TRY(stage_in(c, m, SL_IN0, pre, vol(D, H, W), &dp));
    RTS_TRY(stage_in(c, m, SL_IN1, hr, pix(H, W) * 8, &a));
    RTS_TRY(stage_in(c, m, SL_IN2, ht, pix(H, W) * 8, &b));
    RTS_TRY(stage_in(c, m, SL_IN3, vr, pix(H, W) * 8, &cc));
    RTS_TRY(stage_in(c, m, SL_IN4, vt, pix(H, W) * 8, &dd));
    RTS_TRY(stage_out(c, m, SL_OUT0, out, vol(D, H, W), &dout));
    {
        StageScope sc(c, "cross_aggr");
        launch_cross_aggr(c->stream, (const float *)dp, (float *)dout, (const int *)a, (const int *)b, (const int *)cc,
                          (const int *)dd, H, W, D);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "cross_aggr"));
    RTS_TRY(finish_out(c, m, out, dout, vol(D, H, W)));
    return finish(c, m);
}

rts_status rts_disp_refinement(rts_ctx *ctx, rts_mem m, uint8_t *disp, const int *horz, const int *vert, int H, int W,
                               int D) {
    PROLOGUE(ctx);
    RTS_TRY(check_dims(c, D, H, W));
    void *dd, *tmp;
    const void *dh, *dv;
    RTS_TRY(stage_inout(c, m, SL_IN0, disp, pix(H, W), &dd));
    RTS_TRY(stage_in(c, m, SL_IN1, horz, pix(H, W) * 8, &dh));
    RTS_TRY(stage_in(c, m, SL_IN2, vert, pix(H, W) * 8, &dv));
    RTS_TRY(scratch(c, SL_TMP0, pix(H, W), &tmp));
    {
        StageScope sc(c, "disp_refine");
        launch_disp_refine(c->stream, (const uint8_t *)dd, (uint8_t *)tmp, (const int *)dh, (const int *)dv, H, W, D);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "disp_refine"));
    if (m == RTS_DEVICE) {
        RTS_CU(c, cudaMemcpyAsync(disp, tmp, pix(H, W), cudaMemcpyDeviceToDevice, c->stream));
        return RTS_OK;
    }
    RTS_TRY(finish_out(c, m, disp, tmp, pix(H, W)));
    return finish(c, m);
}

rts_status rts_medianFilt(rts_ctx *ctx, rts_mem m, uint8_t *image, int H, int W, int ch, int k) {
    PROLOGUE(ctx);
    RTS_TRY(check_img(c, H, W));
    if (!image) return bad(c, "null image");
    if (ch != 1 && ch != 3) return bad(c, "channels must be 1 or 3");
    if (!median_ksize_ok(k)) return bad(c, "maskSize must be odd, 3..15");
    const size_t n = pix(H, W) * ch;
    void *di, *tmp;
    RTS_TRY(stage_inout(c, m, SL_IN0, image, n, &di));
    RTS_TRY(scratch(c, SL_TMP0, n, &tmp));
    {
        StageScope sc(c, "median");
        launch_median(c->stream, (const uint8_t *)di, (uint8_t *)tmp, H, W, ch, k);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "median"));
    if (m == RTS_DEVICE) {
        RTS_CU(c, cudaMemcpyAsync(image, tmp, n, cudaMemcpyDeviceToDevice, c->stream));
        return RTS_OK;
    }
    RTS_TRY(finish_out(c, m, image, tmp, n));
    return finish(c, m);
}

rts_status rts_calcProxWeight(rts_ctx *ctx, rts_mem m, float *pw, float gamma_p, int rad) {
    PROLOGUE(ctx);
    if (!pw || rad < 0 || rad > 128) return bad(c, "bad proximity-weight arguments");
    const int area = (2 * rad + 1) * (2 * rad + 1);
    std::vector<float> h(area);
    host_prox_weight(h.data(), gamma_p, rad);
    if (m == RTS_HOST) {
        memcpy(pw, h.data(), area * sizeof(float));
        return RTS_OK;
    }
    RTS_CU(c, cudaMemcpyAsync(pw, h.data(), area * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    RTS_CU(c, cudaStreamSynchronize(c->stream));
    return RTS_OK;
}

rts_status rts_computeWeights(rts_ctx *ctx, rts_mem m, float *w, const float *pw, const uint8_t *lab, float gamma_s,
                              int H, int W, int r) {
    PROLOGUE(ctx);
    RTS_TRY(check_img(c, H, W));
    if (r < 0 || r >= H || r >= W || r > 128) return bad(c, "weight radius out of range");
    const size_t area = (size_t)(2 * r + 1) * (2 * r + 1);
    if ((size_t)W * area >= (1u << 31)) return bad(c, "weight window too large for this width");
    const float *g;
    RTS_TRY(lab_weight_lut(c, gamma_s, &g));
    const void *dl, *dpw;
    void *dw;
    RTS_TRY(stage_in(c, m, SL_IN0, lab, pix(H, W) * 3, &dl));
    RTS_TRY(stage_in(c, m, SL_IN1, pw, area * 4, &dpw));
    RTS_TRY(stage_out(c, m, SL_OUT0, w, pix(H, W) * area * 4, &dw));
    {
        StageScope sc(c, "compute_weights");
        launch_compute_weights(c->stream, (const uint8_t *)dl, (const float *)dpw, g, (float *)dw, H, W, r);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "compute_weights"));
    RTS_TRY(finish_out(c, m, w, dw, pix(H, W) * area * 4));
    return finish(c, m);
}

rts_status rts_calcAWCostL2R(rts_ctx *ctx, rts_mem m, const float *wr, const float *wt, const float *cost,
                             float *newCost, int H, int W, int D, int r) {
    PROLOGUE(ctx);
    RTS_TRY(check_dims(c, D, H, W));
    if (r < 0 || r >= H || r >= W) return bad(c, "window radius out of range");
    const size_t area = (size_t)(2 * r + 1) * (2 * r + 1);
    const void *a, *b, *dc;
    void *dout;
    RTS_TRY(stage_in(c, m, SL_IN0, wr, pix(H, W) * area * 4, &a));
    RTS_TRY(stage_in(c, m, SL_IN1, wt, pix(H, W) * area * 4, &b));
    RTS_TRY(stage_in(c, m, SL_IN2, cost, vol(D, H, W), &dc));
    RTS_TRY(stage_out(c, m, SL_OUT0, newCost, vol(D, H, W), &dout));
    {
        StageScope sc(c, "aw_l2r");
        launch_aw_l2r_weights(c->stream, (const float *)a, (const float *)b, (const float *)dc, (float *)dout, H, W, D,
                              r);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "aw_l2r"));
    RTS_TRY(finish_out(c, m, newCost, dout, vol(D, H, W)));
    return finish(c, m);
}

rts_status rts_calcAWCostR2L(rts_ctx *ctx, rts_mem m, const float *wr, const float *wt, float *cost, int H, int W,
                             int D, int r) {
    PROLOGUE(ctx);
    RTS_TRY(check_dims(c, D, H, W));
    if (r < 0 || r >= H || r + D > W) return bad(c, "window radius out of range");
    const size_t area = (size_t)(2 * r + 1) * (2 * r + 1);
    const void *a, *b;
    void *dc, *tmp;
    RTS_TRY(stage_in(c, m, SL_IN0, wr, pix(H, W) * area * 4, &a));
    RTS_TRY(stage_in(c, m, SL_IN1, wt, pix(H, W) * area * 4, &b));
    RTS_TRY(stage_inout(c, m, SL_IN2, cost, vol(D, H, W), &dc));
    RTS_TRY(scratch(c, SL_TMP0, vol(D, H, W), &tmp));
    {
        StageScope sc(c, "aw_r2l");
        launch_aw_r2l_weights(c->stream, (const float *)a, (const float *)b, (const float *)dc, (float *)tmp, H, W, D,
                              r);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "aw_r2l"));
    if (m == RTS_DEVICE) {
        RTS_CU(c, cudaMemcpyAsync(cost, tmp, vol(D, H, W), cudaMemcpyDeviceToDevice, c->stream));
        return RTS_OK;
    }
    RTS_TRY(finish_out(c, m, cost, tmp, vol(D, H, W)));
    return finish(c, m);
}

// ---- disparity ---------------------------------------------------------------

rts_status rts_WTA(rts_ctx *ctx, rts_mem m, const float *cost, uint8_t *win, int H, int W, int D) {
    PROLOGUE(ctx);
    return wta(c, m, cost, win, H, W, D, 0);
}

rts_status rts_WTA_NCC(rts_ctx *ctx, rts_mem m, const float *cost, uint8_t *win, int H, int W, int D) {
    PROLOGUE(ctx);
    return wta(c, m, cost, win, H, W, D, 1);
}

rts_status rts_cross_check(rts_ctx *ctx, rts_mem m, const uint8_t *dl, const uint8_t *dr, uint8_t *mask, int H,
                           int W) {
    PROLOGUE(ctx);
    RTS_TRY(check_img(c, H, W));
    const void *a, *b;
    void *dm;
    RTS_TRY(stage_in(c, m, SL_IN0, dl, pix(H, W), &a));
    RTS_TRY(stage_in(c, m, SL_IN1, dr, pix(H, W), &b));
    RTS_TRY(stage_out(c, m, SL_OUT0, mask, pix(H, W), &dm));
    {
        StageScope sc(c, "cross_check");
        launch_cross_check(c->stream, (const uint8_t *)a, (const uint8_t *)b, (uint8_t *)dm, H, W);
        count_launch(c);
    }
    RTS_TRY(check_launch(c, "cross_check"));
    RTS_TRY(finish_out(c, m, mask, dm, pix(H, W)));
    return finish(c, m);
}

}  // extern "C"
