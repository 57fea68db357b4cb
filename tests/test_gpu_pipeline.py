"""GPU parity of the whole-pair pipeline (rts_pipeline_run) against the C
oracle's pipeline and the reference-made golden fixtures."""
import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


def synth(seed, W, H, D, rects, planes=0, sigma=2.0):
    import rtstereo_gb300 as R
    L, Rr, _ = R.synth_pair(seed, W, H, D, rects, planes, sigma, min(4, D - 1))
    return L, Rr


def run_both(ctx, oracle_mod, L, Rr, want_cost=False, **kw):
    import rtstereo_gb300 as R
    O = oracle_mod
    rgb = lambda a: np.ascontiguousarray(np.repeat(a[:, :, None], 3, axis=2))
    Lc, Rc = rgb(L), rgb(Rr)
    lab = (R.rgb_to_lab(Lc), R.rgb_to_lab(Rc))
    p = R.params(**kw)
    g = ctx.pipeline(p, L, Rr, Lc, Rc, *lab, want_cost=want_cost)
    op = O.params(cost1=p.cost1, cost2=p.cost2, aggr=p.aggr, lambda1=p.lambda1, lambda2=p.lambda2, D=p.disp_range,
                  census_hrad=p.census_hrad, census_wrad=p.census_wrad, rank_rad=p.rank_rad, ncc_hrad=p.ncc_hrad,
                  ncc_wrad=p.ncc_wrad, box_rad=p.box_rad, aw_rad=p.aw_rad, aw_gamma_s=p.aw_gamma_s,
                  aw_gamma_p=p.aw_gamma_p, cross_L=p.cross_arm, cross_tau=p.cross_tau, ad_trunc=p.ad_trunc,
                  right_view=p.right_view, box_inplace=0)
    o = O.pipeline(op, L, Rr, Lc, Rc, *lab, want_cost=want_cost)
    return g, o


def assert_same(g, o):
    assert bits_equal(g[0], o[0]), "left disparity"
    assert bits_equal(g[1], o[1]), "right disparity"
    assert bits_equal(g[2], o[2]), "cross-check mask"
    if g[3] is not None:
        assert bits_equal(g[3], o[3]), "left cost volume"


def test_config0_ad_census_cross(ctx, oracle_mod):
    # 384x288 random-dot pair, D=16, AD(trunc 24)+census 9x7, cross-based (17, 20), WTA, cross check
    L, Rr = synth(0xC0, 384, 288, 16, 6)
    g, o = run_both(ctx, oracle_mod, L, Rr, disp_range=16)
    assert_same(g, o)
    assert g[2].mean() > 0.5  # most pixels pass the left-right check on this pair


@pytest.mark.parametrize("W,H,D", [(37, 23, 16), (64, 17, 64), (130, 9, 128)])
@pytest.mark.parametrize("aggr", [0, 1, 3])
def test_cost_aggregation_matrix(ctx, oracle_mod, W, H, D, aggr):
    L, Rr = synth(W * H + D, W, H, D, 3)
    for c1, c2 in ((1, 3), (2, 3), (3, 0), (1, 0), (4, 0), (4, 3), (2, 4)):
        g, o = run_both(ctx, oracle_mod, L, Rr, want_cost=True, disp_range=D, cost1=c1, cost2=c2, aggr=aggr,
                        rank_rad=3, box_rad=2)
        if 4 in (c1, c2) and c2 != 0:
            # CombineCost of non-integer LoG differences uses the device expf
            # (the C library's expf is applied through host tables only to
            # integer costs): 1e-4 relative on costs, near-ties may flip.
            np.testing.assert_allclose(g[3], o[3], rtol=1e-4, atol=1e-6)
            assert (g[0] == o[0]).mean() > 0.99
        else:
            assert_same(g, o)


@pytest.mark.parametrize("W,H,D,rad", [(70, 19, 48, 4), (33, 9, 16, 1), (96, 40, 32, 8), (45, 30, 40, 3),
                                       (150, 23, 130, 8), (40, 11, 34, 5), (72, 9, 64, 1), (120, 60, 68, 8),
                                       (100, 40, 96, 2)])
@pytest.mark.parametrize("c1,c2", [(1, 3), (3, 0), (5, 0)])
def test_box_fused_matches_oracle(ctx, oracle_mod, W, H, D, rad, c1, c2):
    # without a cost volume out the box runs as one box + arg-min pass (arg-max for NCC);
    # even D above 32 takes the disparity-pair kernel (ragged last block at D = 34, 130),
    # whose inner tiles arrive by TMA when D is a multiple of 4 (48, 40, 64, 68, 96)
    L, Rr = synth(W * 7 + H + rad, W, H, D, 3)
    g, o = run_both(ctx, oracle_mod, L, Rr, disp_range=D, cost1=c1, cost2=c2, aggr=1, box_rad=rad, ncc_hrad=2,
                    ncc_wrad=2)
    assert_same(g, o)


@pytest.mark.parametrize("W,H,D,rank", [(96, 40, 32, 3), (70, 33, 24, 7), (150, 21, 64, 2)])
def test_rank_census_cross_views(ctx, oracle_mod, W, H, D, rank):
    # rank differences combined with census, cross-based: the view kernels take the
    # ranks from the per-pixel records
    L, Rr = synth(W + 3 * H + rank, W, H, D, 4)
    g, o = run_both(ctx, oracle_mod, L, Rr, disp_range=D, cost1=2, cost2=3, aggr=3, rank_rad=rank)
    assert_same(g, o)


@pytest.mark.parametrize("W,H,D", [(19, 5, 8), (45, 12, 40), (160, 30, 136), (300, 9, 200), (80, 70, 72)])
@pytest.mark.parametrize("gray", [True, False])
def test_cross_views_shapes(ctx, oracle_mod, W, H, D, gray):
    # the cross-based view kernels on disparity ranges that are not multiples of 32
    # (and above 128: eight 32-disparity chunks per lane), tiny and tall images, with
    # and without colour images
    import rtstereo_gb300 as R
    O = oracle_mod
    L, Rr = synth(W * 5 + H + D, W, H, D, 3)
    Lc, Rc = R.gray_to_rgb(L), R.gray_to_rgb(Rr)
    p = R.params(disp_range=D)
    g = ctx.pipeline(p, L, Rr) if gray else ctx.pipeline(p, L, Rr, Lc, Rc)
    o = O.pipeline(O.params(D=D, cross_L=p.cross_arm, cross_tau=p.cross_tau), L, Rr, Lc, Rc)
    assert_same(g, o)


def test_ncc_box(ctx, oracle_mod):
    # the reference's commented-out NCC path: NCC -> box -> WTA_NCC (seq/Main.cpp:287-289)
    L, Rr = synth(77, 96, 40, 32, 4)
    g, o = run_both(ctx, oracle_mod, L, Rr, want_cost=True, disp_range=32, cost1=5, cost2=0, aggr=1, ncc_hrad=3,
                    ncc_wrad=3, box_rad=4)
    assert_same(g, o)


@pytest.mark.parametrize("W,H,D,rad", [(48, 40, 16, 16), (33, 21, 8, 5)])
def test_adaptive_weight_pipeline(ctx, oracle_mod, W, H, D, rad):
    L, Rr = synth(W + H, W, H, D, 3)
    g, o = run_both(ctx, oracle_mod, L, Rr, want_cost=True, disp_range=D, cost1=1, cost2=3, aggr=2, aw_rad=rad)
    assert_same(g, o)


@pytest.mark.parametrize("prec", [0, 1])
def test_cross_views_longest_arm_wide_disparity(ctx, oracle_mod, prec):
    """The fused cross-based views at the longest arm they take (23: the largest
    vertical ring, 72 rows, and eight 32-disparity chunks per lane for D = 200),
    against the oracle; the FP16 form against the plain one."""
    import rtstereo_gb300 as R
    L, Rr = synth(0x23, 224, 40, 200, 4, 1)
    if prec == 0:
        g, o = run_both(ctx, oracle_mod, L, Rr, disp_range=200, aggr=3, cross_arm=23)
        assert_same(g, o)
    else:
        a = ctx.pipeline(R.params(disp_range=200, aggr=3, cross_arm=23), L, Rr)
        b = ctx.pipeline(R.params(disp_range=200, aggr=3, cross_arm=23, precision=R.PREC_F16), L, Rr)
        assert (a[0] == b[0]).mean() > 0.99


def test_fused_paths_match_oracle(ctx, oracle_mod):
    # no cost output requested: the fused kernels run where they exist
    for kw in (dict(disp_range=16, aggr=3), dict(disp_range=64, aggr=3), dict(disp_range=32, aggr=2, aw_rad=7),
               dict(disp_range=80, aggr=2, aw_rad=16), dict(disp_range=100, aggr=3, cost1=3, cost2=1),
               dict(disp_range=40, aggr=3, cost1=2, cost2=3, rank_rad=2), dict(disp_range=24, aggr=2, cost1=3, cost2=0),
               dict(disp_range=24, aggr=1, box_rad=4), dict(disp_range=48, aggr=0)):
        L, Rr = synth(kw["disp_range"], 160, 50, kw["disp_range"], 5, 1)
        g, o = run_both(ctx, oracle_mod, L, Rr, **kw)
        assert_same(g, o)


@pytest.mark.parametrize("W,H,D", [(96, 40, 32), (200, 13, 130)])
def test_fused_log_census_volume_equals_modules(ctx, W, H, D):
    """The one-pass LoG + census volume is the composed modules' volume bit for
    bit (convolveImage, pixelBasedCostL2R_Float, census + Hamming, combineCost)."""
    import rtstereo_gb300 as R
    L, Rr = synth(W * 3 + D, W, H, D, 4)
    p = R.params(cost1=4, cost2=3, aggr=3, disp_range=D, right_view=0)
    got = ctx.pipeline(p, L, Rr, want_cost=True)
    c1 = ctx.pixelBasedCostL2R_Float(ctx.convolveImage(L), ctx.convolveImage(Rr), D)
    c2 = ctx.calcHammingDist(ctx.calcCensusTrans(L), ctx.calcCensusTrans(Rr), D)
    cc = ctx.combineCost(c1, c2, 10.0, 10.0)
    # the pipeline's returned volume is the aggregated one; compare the costs through
    # the modules' aggregation of the same volume
    h, v = ctx.findCross(R.gray_to_rgb(L))
    ht, vt = ctx.findCross(R.gray_to_rgb(Rr))
    agg = ctx.cross_stereo_aggregation(ctx.aggregate_cost_horizontal(cc), h, ht, v, vt)
    assert bits_equal(got[3], agg)


@pytest.mark.parametrize("W,H,D", [(300, 40, 256), (260, 33, 200), (180, 20, 130)])
@pytest.mark.parametrize("c1,c2", [(1, 3), (3, 0)])
def test_cross_wide_disparity_ranges(ctx, oracle_mod, W, H, D, c1, c2):
    """Disparity ranges above 128 on the cross-based views: eight 32-disparity
    chunks per lane in the vertical kernel, a partial last chunk; AD + census on
    float segments, census alone on integer segments."""
    L, Rr = synth(W + H + D, W, H, D, 3)
    g, o = run_both(ctx, oracle_mod, L, Rr, disp_range=D, cost1=c1, cost2=c2, aggr=3)
    assert_same(g, o)


@pytest.mark.parametrize("W,H,D", [(1, 1, 1), (5, 1, 3), (1, 7, 1), (2, 2, 2), (3, 5, 3)])
@pytest.mark.parametrize("aggr", [0, 1, 2, 3])
def test_degenerate_shapes(ctx, oracle_mod, W, H, D, aggr):
    """Single rows, single columns, D = W, windows reduced to the image: the
    pipeline (fused or composed, as it chooses) equals the oracle."""
    rng = np.random.default_rng(W * 100 + H * 10 + D + aggr)
    L = rng.integers(0, 256, (H, W), dtype=np.uint8)
    Rr = rng.integers(0, 256, (H, W), dtype=np.uint8)
    g, o = run_both(ctx, oracle_mod, L, Rr, disp_range=D, cost1=1, cost2=0, aggr=aggr, box_rad=0, aw_rad=0,
                    cross_arm=3)
    assert_same(g, o)


@pytest.mark.parametrize("c1,c2", [(4, 3), (4, 0), (2, 0)])
def test_volume_views_equal_composed_modules(ctx, c1, c2):
    """Cross-based views over a precomputed volume (LoG, rank alone) give the
    disparities of the composed module path on the same volume."""
    import rtstereo_gb300 as R
    L, Rr = synth(c1 * 10 + c2, 160, 48, 48, 5, 1)
    p = R.params(cost1=c1, cost2=c2, aggr=3, disp_range=48, rank_rad=3)
    views = ctx.pipeline(p, L, Rr)
    composed = ctx.pipeline(p, L, Rr, want_cost=True)
    for a, b in zip(views[:3], composed[:3]):
        assert bits_equal(a, b)


@pytest.mark.parametrize("c1", [1, 3])
@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("W,H,D", [(160, 50, 64), (300, 9, 200), (45, 12, 40)])
def test_integer_cost_cross_exact_in_both_forms(ctx, oracle_mod, c1, prec, W, H, D):
    """Census alone or truncated AD alone: the row segments are stored as exact
    u16 integers and summed as integers, so the FP16 form is bit-exact as well."""
    import rtstereo_gb300 as R
    O = oracle_mod
    L, Rr = synth(W + D + c1, W, H, D, 4, 1)
    Lc, Rc = np.repeat(L[:, :, None], 3, 2).copy(), np.repeat(Rr[:, :, None], 3, 2).copy()
    g = ctx.pipeline(R.params(cost1=c1, cost2=0, disp_range=D, precision=prec), L, Rr)
    o = O.pipeline(O.params(cost1=c1, cost2=0, D=D), L, Rr, Lc, Rc)
    assert bits_equal(g[0], o[0]) and bits_equal(g[1], o[1]) and bits_equal(g[2], o[2])


@pytest.mark.parametrize("W,H,D,rad", [(70, 9, 30, 5), (40, 20, 13, 16), (130, 7, 64, 1), (200, 12, 128, 3),
                                       (72, 40, 66, 16)])
def test_fused_adaptive_weight_shapes(ctx, oracle_mod, W, H, D, rad):
    """The fused adaptive-weight kernels (plain and pipelined tap rows) on colour
    inputs: disparity ranges that are not multiples of 4 (word-wise cost copies)
    or span two 64-disparity chunks, windows taller than the image, one-row
    windows, widths that are not multiples of the 64-pixel tile."""
    import rtstereo_gb300 as R
    O = oracle_mod
    L, Rr = synth(W * 7 + D, W, H, D, 3)
    rng = np.random.default_rng(W + H)
    Lc = np.ascontiguousarray(np.stack([L, rng.integers(0, 256, (H, W), dtype=np.uint8), 255 - L], -1))
    Rc = np.ascontiguousarray(np.stack([Rr, rng.integers(0, 256, (H, W), dtype=np.uint8), 255 - Rr], -1))
    lab = (R.rgb_to_lab(Lc), R.rgb_to_lab(Rc))
    p = R.params(disp_range=D, aggr=2, aw_rad=rad)
    g = ctx.pipeline(p, L, Rr, Lc, Rc, *lab)
    o = O.pipeline(O.params(D=D, aggr=2, aw_rad=rad), L, Rr, Lc, Rc, *lab)
    assert bits_equal(g[0], o[0]) and bits_equal(g[1], o[1]) and bits_equal(g[2], o[2])


@pytest.mark.parametrize("name,c1,c2,ag,D", [("pipe_ad_census_cross", 1, 3, 3, 16),
                                              ("pipe_rank_census_aw", 2, 3, 2, 6)])
def test_golden_pipelines(ctx, golden, name, c1, c2, ag, D):
    """Against the pipelines composed from the reference's own functions."""
    import rtstereo_gb300 as R
    L, Rr = golden[f"{name}/L"], golden[f"{name}/R"]
    H, W = L.shape
    rgb = lambda a: np.ascontiguousarray(np.repeat(a[:, :, None], 3, axis=2))
    Lc, Rc = rgb(L), rgb(Rr)
    p = R.params(cost1=c1, cost2=c2, aggr=ag, disp_range=D, aw_rad=16 if min(H, W) > 16 else 5)
    dl, dr, mk, _ = ctx.pipeline(p, L, Rr, Lc, Rc, R.rgb_to_lab(Lc), R.rgb_to_lab(Rc))
    assert bits_equal(dl, golden[f"{name}/disp_left"])
    assert bits_equal(dr, golden[f"{name}/disp_right"])
    assert bits_equal(mk, golden[f"{name}/mask"])


def test_golden_modules(ctx, golden):
    """Module entry points against the reference's own outputs."""
    L, Rr, Lc, Rc = golden["img/L"], golden["img/R"], golden["img/Lc"], golden["img/Rc"]
    D = 16
    assert bits_equal(ctx.pixelBasedCostL2R_Color(Lc, Rc, D, 0, 24.0), golden["L2R_Color_trunc24/n0"])
    assert bits_equal(ctx.pixelBasedR2L_Color(Lc, Rc, D, 1), golden["R2L_Color/n1"])
    bl, br = ctx.calcCensusTrans(L), ctx.calcCensusTrans(Rr)
    assert bits_equal(bl, golden["census4x3/L"])
    assert bits_equal(ctx.calcHammingDist(bl, br, D), golden["hamming4x3"])
    cc = ctx.combineCost(golden["L2R_Color_trunc24/n0"], golden["hamming4x3"], 10.0, 10.0)
    assert bits_equal(cc, golden["combine/10_10"])
    pre = ctx.aggregate_cost_horizontal(cc)
    assert bits_equal(pre, golden["prefix"])
    h, v = ctx.findCross(Lc)
    assert bits_equal(h, golden["findCross/Lh"]) and bits_equal(v, golden["findCross/Lv"])
    agg = ctx.cross_stereo_aggregation(pre, golden["findCross/Lh"], golden["findCross/Rh"], golden["findCross/Lv"],
                                       golden["findCross/Rv"])
    assert bits_equal(agg, golden["cross"])
    assert bits_equal(ctx.WTA(agg), golden["WTA/cross"])
    assert bits_equal(ctx.WTA(golden["WTA/ties_in"]), golden["WTA/ties"])
    assert bits_equal(ctx.convolveImage(L), golden["convolveImage/L"])
    assert bits_equal(ctx.calcNCCDispL2R(L, Rr, D, 3, 3, fill=-7.0), golden["ncc3x3"])
    for rad in (3, 7):
        pw = ctx.calcProxWeight(36.0, rad)
        assert bits_equal(pw, golden[f"aw{rad}/prox"])
        wl = ctx.computeWeights(pw, golden["aw/labL"], 7.0, rad)
        wr = ctx.computeWeights(pw, golden["aw/labR"], 7.0, rad)
        assert bits_equal(ctx.calcAWCostL2R(wl, wr, golden["aw/cost"], rad), golden[f"aw{rad}/l2r"])


@pytest.mark.parametrize("W,H,D,rad", [(96, 20, 40, 5), (300, 40, 64, 16), (40, 9, 40, 3), (52, 12, 36, 4)])
def test_fp16_aw_right_view_from_left_volume(ctx, oracle_mod, W, H, D, rad):
    """FP16 form, adaptive weights: the right view's winners are the arg-min of the
    left view's final volume along the diagonals (x + d mod W, d), with the
    reference's carry, in the right view's mirrored raster order."""
    import rtstereo_gb300 as R
    O = oracle_mod
    L, Rr = synth(W + 3 * H + D, W, H, D, 4)
    Lc, Rc = R.gray_to_rgb(L), R.gray_to_rgb(Rr)
    lab = (R.rgb_to_lab(Lc), R.rgb_to_lab(Rc))
    g = ctx.pipeline(R.params(disp_range=D, aggr=2, aw_rad=rad, precision=R.PREC_F16), L, Rr, Lc, Rc, *lab,
                     want_cost=True)
    vol = g[3]
    assert bits_equal(g[1], diag_right_view(O, vol)), "right disparity"
    assert bits_equal(g[0], O.wta(vol)), "left disparity"
    assert bits_equal(g[2], O.cross_check(g[0], g[1])), "cross-check mask"


def diag_right_view(O, vol):
    """The right view's disparities from the left view's final volume: WTA (with
    the carry, in the right view's mirrored raster order) over (x + d mod W, d)."""
    H, W, D = vol.shape
    xm, d = np.arange(W), np.arange(D)
    cols = ((W - 1 - xm)[:, None] + d[None, :]) % W
    return np.ascontiguousarray(O.wta(np.ascontiguousarray(vol[:, cols, d[None, :]]))[:, ::-1])


@pytest.mark.parametrize("kw", [dict(disp_range=64, aggr=3), dict(disp_range=48, aggr=2, aw_rad=16)])
def test_fp16_form_agrees_with_plain(ctx, kw):
    """FP16 storage (fp32 accumulation): most disparities equal the plain form's."""
    import rtstereo_gb300 as R
    L, Rr = synth(kw["disp_range"] + 1, 200, 60, kw["disp_range"], 6, 1)
    Lc, Rc = R.gray_to_rgb(L), R.gray_to_rgb(Rr)
    lab = (R.rgb_to_lab(Lc), R.rgb_to_lab(Rc))
    a = ctx.pipeline(R.params(precision=R.PREC_F32, **kw), L, Rr, Lc, Rc, *lab)
    b = ctx.pipeline(R.params(precision=R.PREC_F16, **kw), L, Rr, Lc, Rc, *lab)
    agree = (a[0] == b[0]).mean()
    assert agree > 0.97, agree


def test_tma_tiles_complete(ctx, oracle_mod):
    """The box and adaptive-weight kernels take their wrap-free tiles by TMA copies
    with a bounded wait: on shapes with many such tiles the results equal the
    oracle's and no wait gave up."""
    L, Rr = synth(0x7A, 160, 48, 64, 4)
    g, o = run_both(ctx, oracle_mod, L, Rr, disp_range=64, cost1=1, cost2=3, aggr=1, box_rad=4)
    assert_same(g, o)
    g, o = run_both(ctx, oracle_mod, L, Rr, want_cost=True, disp_range=64, cost1=1, cost2=3, aggr=2, aw_rad=7)
    assert_same(g, o)
    assert ctx.tma_timeouts() == 0


def test_cached_graph_after_other_table_sizes(ctx, oracle_mod):
    """A cross-based pair replays its captured CUDA graph after a configuration
    with other cost tables (rank + census: first costs up to 255 against AD's
    24) ran in between: the replay must still read live tables."""
    import rtstereo_gb300 as R
    O = oracle_mod
    L, Rr = synth(0x61, 160, 40, 64, 4)
    kw = dict(disp_range=64, aggr=3, cost1=1, cost2=3)
    first = ctx.pipeline(R.params(**kw), L, Rr)
    ctx.pipeline(R.params(disp_range=64, aggr=3, cost1=2, cost2=3, rank_rad=3), L, Rr)
    again = ctx.pipeline(R.params(**kw), L, Rr)
    o = O.pipeline(O.params(D=64), L, Rr, O.gray_to_rgb(L), O.gray_to_rgb(Rr))
    assert_same(first, o)
    assert_same(again, o)


@pytest.mark.parametrize("W,H,D,rad", [(160, 40, 64, 4), (96, 30, 48, 2), (70, 20, 30, 3)])
def test_fp16_box_right_view_from_left_volume(ctx, oracle_mod, W, H, D, rad):
    """FP16 form, box: one aggregation, the right view the WTA of the left view's box
    means along the diagonals (the box + arg-min kernel's own minima over the
    right pixels x - d, or the composed path's volume when it is asked for); D = 30
    (no disparity-pair kernel) keeps the mirrored right view, the plain form's."""
    import rtstereo_gb300 as R
    O = oracle_mod
    L, Rr = synth(W + 7 * H + D, W, H, D, 4)
    Lc, Rc = R.gray_to_rgb(L), R.gray_to_rgb(Rr)
    kw = dict(disp_range=D, aggr=1, box_rad=rad, cost1=1, cost2=3)
    plain = ctx.pipeline(R.params(**kw), L, Rr, Lc, Rc, want_cost=True)
    f16 = ctx.pipeline(R.params(precision=R.PREC_F16, **kw), L, Rr, Lc, Rc)
    f16c = ctx.pipeline(R.params(precision=R.PREC_F16, **kw), L, Rr, Lc, Rc, want_cost=True)
    assert bits_equal(f16[0], plain[0]) and bits_equal(f16c[0], plain[0]), "left disparity"
    assert bits_equal(f16c[3], plain[3]), "box means"
    if D % 2 == 0 and D > 32:
        want_r = diag_right_view(O, plain[3])
    else:
        want_r = plain[1]
    assert bits_equal(f16[1], want_r), "right disparity (box + arg-min kernel)"
    assert bits_equal(f16c[1], diag_right_view(O, plain[3])), "right disparity (composed path)"
    assert bits_equal(f16[2], O.cross_check(f16[0], f16[1])), "cross-check mask"
