// rts_pipeline.cpp -- whole-pair pipeline (seq/Main.cpp:180-257 for the left
// view; the right view as flip(L2R(flip R, flip L)); then cross_check).
//
// Two execution paths share one entry point:
//   * fused paths (k_pipe.cu) for the configurations the pipeline is built
//     around: cross-based aggregation (cost -> running sum -> row segments in
//     one kernel, vertical sums + WTA in the next) and adaptive weights (tiled
//     weighted sums with the weights made on the fly, WTA fused);
//   * a composed path that chains the module kernels, for every other
//     combination of costs and aggregations.
// Both keep the reference's per-entry arithmetic, so they agree bit for bit.
#include <string.h>

#include <vector>

#include "rts_internal.h"
#include "rts_pipe.h"
#include "rts_views.h"

using namespace rts;

namespace rts {

// seq/Main.cpp:113-117, the 5x5 LoG mask the reference driver convolves with
static const float kLog5x5[25] = {0.0239f, 0.046f,   0.0499f,  0.046f,   0.0239f,  0.046f,  0.0061f,
                                  -0.0923f, 0.0061f, 0.046f,   0.0499f,  -0.0923f, -0.3182f, -0.0923f,
                                  0.0499f,  0.046f,  0.0061f,  -0.0923f, 0.0061f,  0.046f,   0.0239f,
                                  0.046f,   0.0499f, 0.046f,   0.0239f};

rts_status validate_params(rts_ctx *c, const rts_params &p, int H, int W) {
    auto bad = [&](const char *m) { return set_error(c, RTS_ERR_INVALID_ARG, m); };
    if (H <= 0 || W <= 0) return bad("image sizes must be positive");
    const int D = p.disp_range;
    if (D <= 0 || D > kMaxDisp || D > W) return bad("disp_range must be in 1..256 and <= width");
    if (p.cost1 < RTS_COST_AD || p.cost1 > RTS_COST_NCC) return bad("cost1 must be 1..5");
    if (p.cost2 < RTS_COST_NONE || p.cost2 > RTS_COST_LOG) return bad("cost2 must be 0..4");
    if (p.cost1 == RTS_COST_NCC && p.cost2 != RTS_COST_NONE) return bad("NCC is a single (similarity) cost");
    if (p.aggr < RTS_AGGR_NONE || p.aggr > RTS_AGGR_CROSS) return bad("aggr must be 0..3");
    if (p.precision != RTS_PREC_F32 && p.precision != RTS_PREC_F16) return bad("precision must be F32 or F16");
    const bool census = p.cost1 == RTS_COST_CENSUS || p.cost2 == RTS_COST_CENSUS;
    if (census && (p.census_hrad < 0 || p.census_wrad < 0 || p.census_hrad >= H || p.census_wrad >= W ||
                   census_words(p.census_hrad, p.census_wrad) == 0))
        return bad("census window out of range (at most 256 bits)");
    const bool rank = p.cost1 == RTS_COST_RANK || p.cost2 == RTS_COST_RANK;
    if (rank && (p.rank_rad < 0 || p.rank_rad >= H || p.rank_rad >= W)) return bad("rank radius out of range");
    const bool log = p.cost1 == RTS_COST_LOG || p.cost2 == RTS_COST_LOG;
    if (log && (H < 3 || W < 3)) return bad("LoG needs at least 3x3 pixels");
    if (p.cost1 == RTS_COST_NCC && (p.ncc_hrad < 0 || p.ncc_wrad < 0 || p.ncc_hrad >= H || p.ncc_wrad + D > W))
        return bad("NCC radii out of range");
    if (p.aggr == RTS_AGGR_BOX && (p.box_rad < 0 || p.box_rad >= H || p.box_rad >= W)) return bad("box radius out of range");
    if (p.aggr == RTS_AGGR_AW && (p.aw_rad < 0 || p.aw_rad >= H || p.aw_rad >= W || p.aw_rad > 64))
        return bad("adaptive-weight radius out of range");
    if (p.aggr == RTS_AGGR_CROSS && (p.cross_arm < 0 || p.cross_arm > 64)) return bad("cross arm length must be 0..64");
    if (p.cost2 != RTS_COST_NONE && (p.lambda1 == 0.f || p.lambda2 == 0.f)) return bad("lambdas must be non-zero");
    if (p.median_ksize != 0 && (p.aggr != RTS_AGGR_CROSS || !median_ksize_ok(p.median_ksize)))
        return bad("median_ksize must be 0, or odd in 3..15 with cross-based aggregation");
    return RTS_OK;
}

// view-ordered inputs (for the right view: mirrored right image as reference,
// mirrored left image as target)
struct ViewIn {
    const uint8_t *gref, *gtar, *cref, *ctar, *lref, *ltar;
};

// one matching cost into `out` (seq/Main.cpp:180-231)
static rts_status one_cost(rts_ctx *c, const rts_params &p, int which, bool trunc_ad, int H, int W, const ViewIn &v,
                           float *out, int aux_slot) {
    const int D = p.disp_range;
    cudaStream_t s = c->stream;
    const size_t np = (size_t)H * W;
    switch (which) {
    case RTS_COST_AD:
        launch_ad_color(s, v.cref, v.ctar, out, D, H, W, 1, trunc_ad ? 1 : 0, p.ad_trunc, 0);
        count_launch(c);
        return RTS_OK;
    case RTS_COST_RANK: {
        void *aux;
        RTS_TRY(scratch(c, aux_slot, np * 2, &aux));
        uint8_t *a = (uint8_t *)aux, *b = a + np;
        launch_rank(s, v.gref, a, p.rank_rad, H, W);
        launch_rank(s, v.gtar, b, p.rank_rad, H, W);
        launch_ad_gray(s, a, b, out, D, H, W, 1);
        count_launch(c, 3);
        return RTS_OK;
    }
    case RTS_COST_CENSUS: {
        const int nw = census_words(p.census_hrad, p.census_wrad);
        void *codes;
        RTS_TRY(scratch(c, SL_V_CODES, np * nw * 16, &codes));
        uint64_t *a = (uint64_t *)codes, *b = a + np * nw;
        launch_census_codes(s, v.gref, a, p.census_hrad, p.census_wrad, H, W);
        launch_census_codes(s, v.gtar, b, p.census_hrad, p.census_wrad, H, W);
        launch_hamming(s, a, b, out, nw, D, H, W);
        count_launch(c, 3);
        return RTS_OK;
    }
    case RTS_COST_LOG: {
        void *aux, *mask;
        RTS_TRY(scratch(c, aux_slot, np * 8, &aux));
        RTS_TRY(scratch(c, SL_TMP3, sizeof(kLog5x5), &mask));
        RTS_CU(c, cudaMemcpyAsync(mask, kLog5x5, sizeof(kLog5x5), cudaMemcpyHostToDevice, s));
        float *a = (float *)aux, *b = a + np;
        launch_convolve(s, v.gref, a, (const float *)mask, H, W, 2, 2);
        launch_convolve(s, v.gtar, b, (const float *)mask, H, W, 2, 2);
        launch_ad_float(s, a, b, out, D, H, W, 1);
        count_launch(c, 3);
        return RTS_OK;
    }
    case RTS_COST_NCC: {
        void *mean;
        RTS_TRY(scratch(c, SL_V_MEAN, np * 8, &mean));
        float *a = (float *)mean, *b = a + np;
        // cells with a zero denominator stay unwritten (seq/NCCDisparity.cpp:70-71): start from 0
        RTS_CU(c, cudaMemsetAsync(out, 0, np * D * sizeof(float), s));
        launch_window_mean(s, v.gref, a, H, W, p.ncc_hrad, p.ncc_wrad);
        launch_window_mean(s, v.gtar, b, H, W, p.ncc_hrad, p.ncc_wrad);
        launch_ncc(s, v.gref, v.gtar, a, b, out, D, H, W, p.ncc_hrad, p.ncc_wrad);
        count_launch(c, 3);
        return RTS_OK;
    }
    }
    return set_error(c, RTS_ERR_INVALID_ARG, "unknown cost");
}

// cost1 (and cost2 combined, seq/Main.cpp:180-234) into `out` with the module kernels
static rts_status cost_volume_composed(rts_ctx *c, const rts_params &p, int H, int W, const ViewIn &v, float *out) {
    const size_t ne = (size_t)H * W * p.disp_range;
    const int nw = census_words(p.census_hrad, p.census_wrad);
    if (p.cost1 == RTS_COST_LOG && p.cost2 == RTS_COST_CENSUS && nw > 0) {
        // LoG and census terms combined as the volume is written (one pass)
        const size_t np = (size_t)H * W;
        cudaStream_t s = c->stream;
        void *aux, *mask, *codes;
        RTS_TRY(scratch(c, SL_V_AUX, np * 8, &aux));
        RTS_TRY(scratch(c, SL_TMP3, sizeof(kLog5x5), &mask));
        RTS_TRY(scratch(c, SL_V_CODES, np * nw * 16, &codes));
        RTS_CU(c, cudaMemcpyAsync(mask, kLog5x5, sizeof(kLog5x5), cudaMemcpyHostToDevice, s));
        float *la = (float *)aux, *lb = la + np;
        uint64_t *ca = (uint64_t *)codes, *cb = ca + np * nw;
        launch_convolve(s, v.gref, la, (const float *)mask, H, W, 2, 2);
        launch_convolve(s, v.gtar, lb, (const float *)mask, H, W, 2, 2);
        launch_census_codes(s, v.gref, ca, p.census_hrad, p.census_wrad, H, W);
        launch_census_codes(s, v.gtar, cb, p.census_hrad, p.census_wrad, H, W);
        const float *l1, *l2;
        RTS_TRY(combine_luts(c, p.lambda1, p.lambda2, &l1, &l2));
        launch_cost_log_census(s, la, lb, ca, cb, nw, out, p.disp_range, H, W, l1, l2, p.lambda1, p.lambda2);
        count_launch(c, 5);
        return RTS_OK;
    }
    RTS_TRY(one_cost(c, p, p.cost1, p.aggr == RTS_AGGR_CROSS, H, W, v, out, SL_V_AUX));
    if (p.cost2 != RTS_COST_NONE) {
        void *c2v;
        RTS_TRY(scratch(c, SL_V_COST2, ne * 4, &c2v));
        RTS_TRY(one_cost(c, p, p.cost2, false, H, W, v, (float *)c2v, SL_TMP2));
        const float *l1, *l2;
        RTS_TRY(combine_luts(c, p.lambda1, p.lambda2, &l1, &l2));
        launch_combine(c->stream, out, (const float *)c2v, (long)ne, l1, l2, p.lambda1, p.lambda2);
        count_launch(c);
    }
    return RTS_OK;
}

// Composed path for one view: module kernels in the reference's order.
static rts_status view_composed(rts_ctx *c, const rts_params &p, int H, int W, const ViewIn &v, uint8_t *disp,
                                int mirror, float *cost_out, unsigned long long *box_best_r = nullptr) {
    const int D = p.disp_range;
    const size_t np = (size_t)H * W, ne = np * D;
    cudaStream_t s = c->stream;
    void *c1v, *finv = nullptr;
    RTS_TRY(scratch(c, SL_V_COST1, ne * 4, &c1v));
    float *c1 = (float *)c1v;
    const bool box_pass = p.aggr == RTS_AGGR_BOX && !cost_out && box_best_supported(p.box_rad);
    if (box_pass && fast_costs(p)) {
        // AD / census costs of the box pass: one volume pass from per-pixel records
        StageScope sc(c, "cost");
        void *recv;
        RTS_TRY(scratch(c, SL_V_REC, np * 32, &recv));
        uint4 *rr = (uint4 *)recv, *rt = rr + np;
        RTS_TRY(prep_records(c, p, H, W, v.gref, v.cref, rr, nullptr));
        RTS_TRY(prep_records(c, p, H, W, v.gtar, v.ctar, rt, nullptr));
        RTS_TRY(cost_volume_fast(c, p, H, W, rr, rt, c1, 0));
    } else {
        StageScope sc(c, "cost");
        RTS_TRY(one_cost(c, p, p.cost1, p.aggr == RTS_AGGR_CROSS, H, W, v, c1, SL_V_AUX));
        if (p.cost2 != RTS_COST_NONE) {
            void *c2v;
            RTS_TRY(scratch(c, SL_V_COST2, ne * 4, &c2v));
            RTS_TRY(one_cost(c, p, p.cost2, false, H, W, v, (float *)c2v, SL_TMP2));
            const float *l1, *l2;
            RTS_TRY(combine_luts(c, p.lambda1, p.lambda2, &l1, &l2));
            launch_combine(s, c1, (const float *)c2v, (long)ne, l1, l2, p.lambda1, p.lambda2);
            count_launch(c);
        }
    }
    float *fin = c1;
    const int argmax = (p.cost1 == RTS_COST_NCC && p.cost2 == RTS_COST_NONE) ? 1 : 0;
    if (box_pass) {
        // box mean and arg-min in one pass over the volume
        void *raw, *rl, *bestv;
        RTS_TRY(scratch(c, SL_V_RAW, np * 2, &raw));
        RTS_TRY(scratch(c, SL_V_ROWLAST, (size_t)H * 4, &rl));
        RTS_TRY(scratch(c, SL_V_SEG, np * 8, &bestv));
        {
            StageScope sc(c, "box_wta");
            RTS_CU(c, cudaMemsetAsync(rl, 0xff, (size_t)H * 4, s));
            RTS_CU(c, cudaMemsetAsync(bestv, 0xff, np * 8, s));
            // every cost but NCC is >= 0 (absolute differences, distances, 1 - exp(-c/l))
            const bool pos = p.cost1 != RTS_COST_NCC;
            launch_box_best(s, c1, (unsigned long long *)bestv, (uint16_t *)raw, (int *)rl, H, W, D, p.box_rad, argmax,
                            pos ? 1 : 0, box_best_r);
            count_launch(c, 2);
        }
        {
            StageScope sc(c, "wta_fill");
            launch_wta_fill(s, (const uint16_t *)raw, (const int *)rl, disp, H, W, mirror);
            count_launch(c);
        }
        return check_launch(c, "pipeline view");
    }
    if (p.aggr == RTS_AGGR_BOX) {
        StageScope sc(c, "box");
        RTS_TRY(scratch(c, SL_V_SEG, ne * 4, &finv));
        launch_box(s, c1, (float *)finv, H, W, D, p.box_rad);
        count_launch(c);
        fin = (float *)finv;
    } else if (p.aggr == RTS_AGGR_AW) {
        StageScope sc(c, "adaptive_weight");
        const size_t area = (size_t)(2 * p.aw_rad + 1) * (2 * p.aw_rad + 1);
        const float *pw, *g;
        RTS_TRY(prox_weights(c, p.aw_gamma_p, p.aw_rad, &pw));
        RTS_TRY(lab_weight_lut(c, p.aw_gamma_s, &g));
        void *wr, *wt;
        RTS_TRY(scratch(c, SL_TMP0, np * area * 4, &wr));
        RTS_TRY(scratch(c, SL_TMP1, np * area * 4, &wt));
        RTS_TRY(scratch(c, SL_V_SEG, ne * 4, &finv));
        launch_compute_weights(s, v.lref, pw, g, (float *)wr, H, W, p.aw_rad);
        launch_compute_weights(s, v.ltar, pw, g, (float *)wt, H, W, p.aw_rad);
        launch_aw_l2r_weights(s, (const float *)wr, (const float *)wt, c1, (float *)finv, H, W, D, p.aw_rad);
        count_launch(c, 3);
        fin = (float *)finv;
    } else if (p.aggr == RTS_AGGR_CROSS) {
        StageScope sc(c, "cross");
        void *arms;
        RTS_TRY(scratch(c, SL_V_ARMS, np * 8 * 4, &arms));
        int *hr = (int *)arms, *vr = hr + 2 * np, *ht = vr + 2 * np, *vt = ht + 2 * np;
        RTS_TRY(scratch(c, SL_V_SEG, ne * 4, &finv));
        const uint8_t *ar = v.cref, *at = v.ctar;
        if (p.median_ksize) {
            // arms on median-filtered copies; the filter commutes with the mirroring of
            // the right view's images (a symmetric window, replicated borders)
            void *mv;
            RTS_TRY(scratch(c, SL_V_MED, np * 6, &mv));
            launch_median(s, v.cref, (uint8_t *)mv, H, W, 3, p.median_ksize);
            launch_median(s, v.ctar, (uint8_t *)mv + 3 * np, H, W, 3, p.median_ksize);
            count_launch(c, 2);
            ar = (const uint8_t *)mv;
            at = ar + 3 * np;
        }
        launch_find_cross(s, ar, hr, vr, H, W, p.cross_arm, p.cross_tau);
        launch_find_cross(s, at, ht, vt, H, W, p.cross_arm, p.cross_tau);
        launch_prefix_h(s, c1, H, W, D);
        launch_cross_aggr(s, c1, (float *)finv, hr, ht, vr, vt, H, W, D);
        count_launch(c, 4);
        fin = (float *)finv;
    }
    {
        StageScope sc(c, "wta");
        void *raw, *rl;
        RTS_TRY(scratch(c, SL_V_RAW, np * 2, &raw));
        RTS_TRY(scratch(c, SL_V_ROWLAST, (size_t)H * 4, &rl));
        RTS_CU(c, cudaMemsetAsync(rl, 0xff, (size_t)H * 4, s));
        launch_wta_local(s, fin, (uint16_t *)raw, (int *)rl, H, W, D, argmax);
        launch_wta_fill(s, (const uint16_t *)raw, (const int *)rl, disp, H, W, mirror);
        count_launch(c, 2);
    }
    if (cost_out) RTS_CU(c, cudaMemcpyAsync(cost_out, fin, ne * 4, cudaMemcpyDeviceToDevice, s));
    return check_launch(c, "pipeline view");
}

// Fused path for one view (cross-based or adaptive-weight aggregation).
static rts_status view_fused(rts_ctx *c, const rts_params &p, int H, int W, const ViewIn &v, uint8_t *disp,
                             int mirror, float *cost_out) {
    const int D = p.disp_range;
    const size_t np = (size_t)H * W, ne = np * D;
    cudaStream_t s = c->stream;
    const bool half = p.precision == RTS_PREC_F16;
    void *recv, *raw, *rl;
    RTS_TRY(scratch(c, SL_V_REC, np * 32, &recv));
    uint4 *rr = (uint4 *)recv, *rt = rr + np;
    RTS_TRY(scratch(c, SL_V_RAW, np * 2, &raw));
    RTS_TRY(scratch(c, SL_V_ROWLAST, (size_t)H * 4, &rl));
    RTS_CU(c, cudaMemsetAsync(rl, 0xff, (size_t)H * 4, s));
    {
        StageScope sc(c, "prep");
        RTS_TRY(prep_records(c, p, H, W, v.gref, v.cref, rr, nullptr));
        RTS_TRY(prep_records(c, p, H, W, v.gtar, v.ctar, rt, nullptr));
    }
    const bool fast = fast_costs(p);
    const void *vol = nullptr;
    int vol_half = 0;
    {
        StageScope sc(c, "cost");
        void *c1v;
        if (fast) {
            vol_half = half ? 1 : 0;
            RTS_TRY(scratch(c, SL_V_COST1, ne * (half ? 2 : 4), &c1v));
            RTS_TRY(cost_volume_fast(c, p, H, W, rr, rt, c1v, vol_half));
        } else {
            RTS_TRY(scratch(c, SL_V_COST1, ne * 4, &c1v));
            RTS_TRY(cost_volume_composed(c, p, H, W, v, (float *)c1v));
        }
        vol = c1v;
    }
    RTS_TRY(aw_fused(c, p, H, W, vol, vol_half, v.lref, v.ltar, (uint16_t *)raw, (int *)rl, cost_out));
    {
        StageScope sc(c, "wta_fill");
        launch_wta_fill(s, (const uint16_t *)raw, (const int *)rl, disp, H, W, mirror);
        count_launch(c);
    }
    return check_launch(c, "pipeline view");
}

rts_status run_view(rts_ctx *c, const rts_params &p, int H, int W, const ViewIn &v, uint8_t *disp, int mirror,
                    float *cost_out, unsigned long long *box_best_r = nullptr) {
    // the fused kernel also writes the final volume when one is asked for
    if (p.aggr == RTS_AGGR_AW && fused_supported(p, H, W)) return view_fused(c, p, H, W, v, disp, mirror, cost_out);
    return view_composed(c, p, H, W, v, disp, mirror, cost_out, box_best_r);
}

// Cross-based pipeline of one pair over a view table: both views run in the
// same launch of every stage (the right view through mirrored addressing).
static rts_status pipeline_cross_views(rts_ctx *c, const rts_params &p, int H, int W, const uint8_t *lg,
                                       const uint8_t *rg, const uint8_t *lc, const uint8_t *rc, uint8_t *dl,
                                       uint8_t *dr, uint8_t *mask) {
    if (cross_record_costs(p)) {
        // the batched form with one pair: autotuned tiles and a captured graph per shape
        rts_pair pr{W, H, lg, rg, lc, rc, nullptr, nullptr};
        rts_out o{dl, dr, mask, nullptr};
        return batch_views_run(c, 1, &pr, &p, &o);
    }
    const int nv = p.right_view ? 2 : 1;
    const int half = p.precision == RTS_PREC_F16 ? 1 : 0;
    const int Ws[2] = {W, W}, Hs[2] = {H, H}, Ds[2] = {p.disp_range, p.disp_range};
    CrossTune tune;
    ViewBatch b;
    RTS_TRY(plan_views(c, SL_BATCH0, Ws, Hs, Ds, nv, half, tune, &b));
    ViewDesc &v0 = b.views[0];
    v0.gref = lg; v0.gtar = rg; v0.cref = lc; v0.ctar = rc; v0.mirror = 0; v0.disp = dl;
    if (p.median_ksize) {
        // arms on median-filtered copies of the (three-channel) colour images
        const size_t n3 = (size_t)H * W * 3;
        void *mv;
        RTS_TRY(scratch(c, SL_V_MED, n3 * 2, &mv));
        StageScope sc(c, "median");
        launch_median(c->stream, lc, (uint8_t *)mv, H, W, 3, p.median_ksize);
        launch_median(c->stream, rc, (uint8_t *)mv + n3, H, W, 3, p.median_ksize);
        count_launch(c, 2);
        v0.mref = (const uint8_t *)mv;
        v0.mtar = (const uint8_t *)mv + n3;
    }
    if (nv == 2) {
        ViewDesc &v1 = b.views[1];
        v1.gref = rg; v1.gtar = lg; v1.cref = rc; v1.ctar = lc; v1.mirror = 1; v1.disp = dr;
        v0.mask = mask;
        link_pair(&b, 0, 1);
    }
    int has_vol = 0;
    if (!cross_record_costs(p)) {
        // other costs: the module kernels build each view's volume first
        // (the right view from mirrored copies of the images)
        has_vol = 1;
        const size_t np = (size_t)H * W, ne = np * p.disp_range;
        StageScope sc(c, "cost");
        void *vol0;
        RTS_TRY(scratch(c, SL_BATCH2, ne * 4, &vol0));
        ViewIn in0{lg, rg, lc, rc, nullptr, nullptr};
        RTS_TRY(cost_volume_composed(c, p, H, W, in0, (float *)vol0));
        b.views[0].vol = (const float *)vol0;
        if (nv == 2) {
            void *gv, *cv, *vol1;
            RTS_TRY(scratch(c, SL_V_GRAY, np * 2, &gv));
            RTS_TRY(scratch(c, SL_V_LAB, np * 6, &cv));
            uint8_t *fg_r = (uint8_t *)gv, *fg_l = fg_r + np, *fc_r = (uint8_t *)cv, *fc_l = fc_r + 3 * np;
            launch_flip(c->stream, rg, fg_r, H, W, 1, 1);
            launch_flip(c->stream, lg, fg_l, H, W, 1, 1);
            launch_flip(c->stream, rc, fc_r, H, W, 3, 1);
            launch_flip(c->stream, lc, fc_l, H, W, 3, 1);
            count_launch(c, 4);
            RTS_TRY(scratch(c, SL_BATCH3, ne * 4, &vol1));
            ViewIn in1{fg_r, fg_l, fc_r, fc_l, nullptr, nullptr};
            RTS_TRY(cost_volume_composed(c, p, H, W, in1, (float *)vol1));
            b.views[1].vol = (const float *)vol1;
        }
    }
    ViewTable t;
    RTS_TRY(cross_tables(c, p));
    RTS_TRY(upload_views(c, b, tune, nullptr, &t));
    return launch_cross_views(c, p, t, half, has_vol, (!lc || !rc) ? 1 : 0, b.max_d, tune, b.row_last_all,
                              b.row_last_count);
}

// Prepares device inputs for both views and runs them; all pointers device.
rts_status pipeline_device(rts_ctx *c, const rts_params &p, int H, int W, const uint8_t *lg, const uint8_t *rg,
                           const uint8_t *lc, const uint8_t *rc, const uint8_t *ll, const uint8_t *rl, uint8_t *dl,
                           uint8_t *dr, uint8_t *mask, float *cost_out) {
    const size_t np = (size_t)H * W;
    cudaStream_t s = c->stream;
    // the cross-based view kernels read gray images directly when there is no colour
    if (!cost_out && p.aggr == RTS_AGGR_CROSS && cross_fused_supported(p) && cross_record_costs(p))
        return pipeline_cross_views(c, p, H, W, lg, rg, lc && rc ? lc : nullptr, lc && rc ? rc : nullptr, dl, dr,
                                    mask);
    const bool need_lab = p.aggr == RTS_AGGR_AW;
    // the fused kernels read packed colour records even for gray-only costs
    const bool need_rgb = true;
    void *rgbv = nullptr;
    if (need_rgb && (!lc || !rc)) {
        // gray replicated into three channels (seq/Main.cpp:87-90 reads the files as colour)
        RTS_TRY(scratch(c, SL_V_RGB, np * 12, &rgbv));
        uint8_t *a = (uint8_t *)rgbv, *b = a + 3 * np;
        launch_gray_to_rgb(s, lg, a, (long)np);
        launch_gray_to_rgb(s, rg, b, (long)np);
        count_launch(c, 2);
        lc = a;
        rc = b;
    }
    if (!cost_out && p.aggr == RTS_AGGR_CROSS && cross_fused_supported(p))
        return pipeline_cross_views(c, p, H, W, lg, rg, lc, rc, dl, dr, mask);
    // FP16 form, adaptive weights or box: the right view's final costs are the left
    // view's read along diagonals, so one aggregation serves both views.  Not for NCC
    // (an arg-max whose products are not symmetric in the two images).  Adaptive
    // weights and a box whose volume the caller asked for: the final volume, then
    // launch_wta_diag; otherwise the box + arg-min kernel enters the right view's
    // minima itself (even D above 32).
    const bool sym = p.cost1 != RTS_COST_NCC && p.cost2 != RTS_COST_NCC;
    const bool shared_aw = p.aggr == RTS_AGGR_AW && fused_supported(p, H, W);
    const bool box_rv = p.aggr == RTS_AGGR_BOX && !cost_out && box_best_right_supported(p.box_rad, p.disp_range);
    const bool shared_box = p.aggr == RTS_AGGR_BOX && (cost_out || box_rv);
    const bool shared_right = p.right_view && p.precision == RTS_PREC_F16 && sym && (shared_aw || shared_box);
    float *final_vol = cost_out;
    unsigned long long *best_r = nullptr;
    if (shared_right && box_rv) {
        void *bv;
        RTS_TRY(scratch(c, SL_V_FINAL, np * 8, &bv));
        best_r = (unsigned long long *)bv;
        RTS_CU(c, cudaMemsetAsync(best_r, 0xff, np * 8, s));
    } else if (shared_right && !final_vol) {
        void *fv;
        RTS_TRY(scratch(c, SL_V_FINAL, np * p.disp_range * 4, &fv));
        final_vol = (float *)fv;
    }
    {
        StageScope sc(c, "left_view");
        ViewIn v{lg, rg, lc, rc, ll, rl};
        RTS_TRY(run_view(c, p, H, W, v, dl, 0, final_vol, best_r));
    }
    if (!p.right_view) return RTS_OK;
    if (shared_right) {
        void *raw, *rlast;
        {
            StageScope sc(c, "right_view");
            RTS_TRY(scratch(c, SL_V_RAW, np * 2, &raw));
            RTS_TRY(scratch(c, SL_V_ROWLAST, (size_t)H * 4, &rlast));
            RTS_CU(c, cudaMemsetAsync(rlast, 0xff, (size_t)H * 4, s));
            if (best_r) launch_best_raw(s, best_r, (uint16_t *)raw, (int *)rlast, H, W, 1);
            else launch_wta_diag(s, final_vol, (uint16_t *)raw, (int *)rlast, H, W, p.disp_range);
            launch_wta_fill(s, (const uint16_t *)raw, (const int *)rlast, dr, H, W, 1);
            count_launch(c, 2);
        }
        StageScope sc(c, "cross_check");
        launch_cross_check(s, dl, dr, mask, H, W);
        count_launch(c);
        return check_launch(c, "pipeline");
    }
    // right view: mirrored copies (a few bytes per pixel next to the D floats per pixel of the view)
    void *gv, *cv = nullptr, *lv = nullptr;
    RTS_TRY(scratch(c, SL_V_GRAY, np * 2, &gv));
    uint8_t *fg_r = (uint8_t *)gv, *fg_l = fg_r + np;
    launch_flip(s, rg, fg_r, H, W, 1, 1);
    launch_flip(s, lg, fg_l, H, W, 1, 1);
    count_launch(c, 2);
    uint8_t *fc_r = nullptr, *fc_l = nullptr, *fl_r = nullptr, *fl_l = nullptr;
    if (need_rgb) {
        // SL_V_RGB may already hold the replicated colour images in its first half
        void *base;
        RTS_TRY(scratch(c, SL_V_RGB, np * 12, &base));
        if (rgbv && base != rgbv) return set_error(c, RTS_ERR_CUDA, "scratch moved");
        cv = base;
        fc_r = (uint8_t *)cv + 6 * np;
        fc_l = fc_r + 3 * np;
        launch_flip(s, rc, fc_r, H, W, 3, 1);
        launch_flip(s, lc, fc_l, H, W, 3, 1);
        count_launch(c, 2);
    }
    if (need_lab) {
        RTS_TRY(scratch(c, SL_V_LAB, np * 6, &lv));
        fl_r = (uint8_t *)lv;
        fl_l = fl_r + 3 * np;
        launch_flip(s, rl, fl_r, H, W, 3, 1);
        launch_flip(s, ll, fl_l, H, W, 3, 1);
        count_launch(c, 2);
    }
    {
        StageScope sc(c, "right_view");
        ViewIn v{fg_r, fg_l, fc_r, fc_l, fl_r, fl_l};
        RTS_TRY(run_view(c, p, H, W, v, dr, 1, nullptr));
    }
    {
        StageScope sc(c, "cross_check");
        launch_cross_check(s, dl, dr, mask, H, W);
        count_launch(c);
    }
    return check_launch(c, "pipeline");
}

}  // namespace rts

extern "C" {

void rts_params_default(rts_params *p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->cost1 = RTS_COST_AD;
    p->cost2 = RTS_COST_CENSUS;
    p->aggr = RTS_AGGR_CROSS;
    p->lambda1 = 10.f;  // seq/Main.cpp:130-131 (LambdaAD, LambdaCensus)
    p->lambda2 = 10.f;
    p->disp_range = 16;
    p->census_hrad = 4;
    p->census_wrad = 3;
    p->rank_rad = 7;
    p->ncc_hrad = 1;
    p->ncc_wrad = 1;
    p->box_rad = 1;
    p->aw_rad = 16;
    p->aw_gamma_s = 7.f;
    p->aw_gamma_p = 36.f;
    p->cross_arm = 17;
    p->cross_tau = 20;
    p->ad_trunc = 24.f;
    p->right_view = 1;
    p->precision = RTS_PREC_F32;
    p->median_ksize = 0;
}

rts_status rts_pipeline_run(rts_ctx *ctx, rts_mem m, const rts_pair *pair, const rts_params *params, rts_out *out) {
    if (!ctx || !pair || !params || !out) return RTS_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> g(ctx->mu);
    rts_ctx *c = ctx;
    if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, RTS_ERR_CUDA, "cudaSetDevice failed");
    const rts_params &p = *params;
    const int H = pair->height, W = pair->width;
    RTS_TRY(validate_params(c, p, H, W));
    if (!pair->left_gray || !pair->right_gray || !out->disp_left) return set_error(c, RTS_ERR_INVALID_ARG, "null image or output");
    if (p.right_view && (!out->disp_right || !out->mask)) return set_error(c, RTS_ERR_INVALID_ARG, "right view needs disp_right and mask");
    if (p.aggr == RTS_AGGR_AW && (!pair->left_lab || !pair->right_lab)) return set_error(c, RTS_ERR_INVALID_ARG, "adaptive weights need Lab images");
    // (the box path keeps f32 volumes in both forms)
    if (out->cost_left && p.precision != RTS_PREC_F32 && !(p.aggr == RTS_AGGR_AW && fused_supported(p, H, W)) &&
        p.aggr != RTS_AGGR_BOX)
        return set_error(c, RTS_ERR_INVALID_ARG,
                         "cost_left: the plain form, or the FP16 form of adaptive weights or box aggregation");
    const size_t np = (size_t)H * W, ne = np * p.disp_range;
    const uint8_t *lg, *rg, *lc = nullptr, *rc = nullptr, *ll = nullptr, *rl = nullptr;
    const void *t;
    RTS_TRY(stage_in(c, m, SL_IN0, pair->left_gray, np, &t)); lg = (const uint8_t *)t;
    RTS_TRY(stage_in(c, m, SL_IN1, pair->right_gray, np, &t)); rg = (const uint8_t *)t;
    if (pair->left_rgb && pair->right_rgb) {
        RTS_TRY(stage_in(c, m, SL_IN2, pair->left_rgb, np * 3, &t)); lc = (const uint8_t *)t;
        RTS_TRY(stage_in(c, m, SL_IN3, pair->right_rgb, np * 3, &t)); rc = (const uint8_t *)t;
    }
    if (p.aggr == RTS_AGGR_AW) {
        RTS_TRY(stage_in(c, m, SL_IN4, pair->left_lab, np * 3, &t)); ll = (const uint8_t *)t;
        RTS_TRY(stage_in(c, m, SL_IN5, pair->right_lab, np * 3, &t)); rl = (const uint8_t *)t;
    }
    uint8_t *dl, *dr = nullptr, *mk = nullptr;
    float *co = nullptr;
    void *o;
    if (m == RTS_DEVICE) {
        dl = out->disp_left;
        dr = out->disp_right;
        mk = out->mask;
        co = out->cost_left;
    } else {
        RTS_TRY(scratch(c, SL_OUT0, np * 3, &o));
        dl = (uint8_t *)o;
        dr = dl + np;
        mk = dr + np;
        if (out->cost_left) {
            RTS_TRY(scratch(c, SL_OUT1, ne * 4, &o));
            co = (float *)o;
        }
    }
    RTS_TRY(pipeline_device(c, p, H, W, lg, rg, lc, rc, ll, rl, dl, dr, mk, co));
    if (m == RTS_HOST) {
        RTS_CU(c, cudaMemcpyAsync(out->disp_left, dl, np, cudaMemcpyDeviceToHost, c->stream));
        if (p.right_view) {
            RTS_CU(c, cudaMemcpyAsync(out->disp_right, dr, np, cudaMemcpyDeviceToHost, c->stream));
            RTS_CU(c, cudaMemcpyAsync(out->mask, mk, np, cudaMemcpyDeviceToHost, c->stream));
        }
        if (co) RTS_CU(c, cudaMemcpyAsync(out->cost_left, co, ne * 4, cudaMemcpyDeviceToHost, c->stream));
        RTS_CU(c, cudaStreamSynchronize(c->stream));
    }
    return RTS_OK;
}

}  // extern "C"
