"""The C oracle against the reference's own seq/ code compiled from its sources
(oracle/_ref, built where the reference tree is present), on seeded inputs of
several sizes.  Skipped on machines without the reference build; the golden
fixtures pin the oracle there."""
import numpy as np
import pytest

from conftest import bits_equal, smooth

oracle = pytest.importorskip("oracle")
if not oracle.have_reference():
    pytest.skip("reference seq/ not built here (oracle/_ref)", allow_module_level=True)

REF = oracle.reflib()
P = oracle.ptr

SIZES = [(7, 9, 1), (23, 37, 16), (31, 48, 32), (12, 64, 64)]


def pair(seed, H, W):
    rng = np.random.default_rng(seed)
    L = smooth(rng.integers(0, 256, (H, W), dtype=np.uint8))
    R = smooth(rng.integers(0, 256, (H, W), dtype=np.uint8))
    Lc = np.ascontiguousarray(np.stack([L, smooth(rng.integers(0, 256, (H, W), dtype=np.uint8)), L], -1))
    Rc = np.ascontiguousarray(np.stack([R, R, smooth(rng.integers(0, 256, (H, W), dtype=np.uint8))], -1))
    return L, R, Lc, Rc


@pytest.mark.parametrize("H,W,D", SIZES)
def test_costs(H, W, D):
    L, R, Lc, Rc = pair(H * W + D, H, W)
    for fn, dirn in (("pixelBasedL2R", 1), ("pixelBasedR2L", -1)):
        o = np.zeros((H, W, D), np.float32)
        getattr(REF, "ref_" + fn)(P(L), P(R), P(o), D, H, W)
        assert bits_equal(oracle.ad_gray(L, R, D, dirn), o)
    for norm in (0, 1):
        for tr in (None, 24.0, 7.5):
            for dirn, fn in ((1, "L2R"), (-1, "R2L")):
                o = np.zeros((H, W, D), np.float32)
                name = "ref_pixelBasedCostL2R_Color" if fn == "L2R" else "ref_pixelBasedR2L_Color"
                if tr is None:
                    getattr(REF, name)(P(Lc), P(Rc), P(o), D, H, W, norm)
                else:
                    getattr(REF, name + "_trunc")(P(Lc), P(Rc), P(o), D, H, W, tr, norm)
                assert bits_equal(oracle.ad_color(Lc, Rc, D, dirn, tr, norm), o)
    if H > 4 and W > 3:
        bl = np.zeros((H, W, 63), np.uint8)
        REF.ref_calcCensusTrans(P(L), P(bl), 4, 3, H, W)
        assert bits_equal(oracle.census(L, 4, 3), bl)
        br = oracle.census(R, 4, 3)
        o = np.zeros((H, W, D), np.float32)
        REF.ref_calcHammingDist(P(bl), P(br), P(o), 4, 3, H, W, D)
        assert bits_equal(oracle.hamming(bl, br, D, 4, 3), o)
    for m in (1, 2):
        if m < min(H, W):
            o = np.zeros((H, W), np.uint8)
            REF.ref_calculateRankFilt(P(L), P(o), m, H, W)
            assert bits_equal(oracle.rank(L, m), o)
    if min(H, W) > 2:
        f = np.zeros((H, W), np.float32)
        REF.ref_convolveImage(P(L), P(f), P(oracle.LOG5x5), H, W, 2, 2)
        assert bits_equal(oracle.convolve(L, oracle.LOG5x5, 2, 2), f)
    if W >= D + 1 and H > 1:
        o = np.full((H, W, D), 3.0, np.float32)
        REF.ref_calcNCCDispL2R(P(L), P(R), P(o), D, H, W, 1, 1)
        assert bits_equal(oracle.ncc(L, R, D, 1, 1, fill=3.0), o)


@pytest.mark.parametrize("H,W,D", SIZES)
def test_aggregation_and_wta(H, W, D):
    L, R, Lc, Rc = pair(7 * H + W + D, H, W)
    c1 = oracle.ad_color(Lc, Rc, D, 1, 24.0, 0)
    c2 = oracle.ad_gray(L, R, D, 1)
    a = c1.copy()
    REF.ref_combineCost(P(a), P(c2.copy()), 10.0, 17.0, H, W, D)
    cc = oracle.combine(c1, c2, 10.0, 17.0)
    assert bits_equal(cc, a)
    for r in (1, 2):
        if r < min(H, W):
            a = cc.copy()
            REF.ref_boxAggregate(P(a), H, W, D, r)
            assert bits_equal(oracle.box(cc, r, inplace=True), a)
    hl = np.zeros((H, W, 2), np.int32)
    vl = np.zeros((H, W, 2), np.int32)
    REF.ref_findCross(P(Lc), P(hl), P(vl), H, W)
    h2, v2 = oracle.find_cross(Lc)
    assert bits_equal(h2, hl) and bits_equal(v2, vl)
    ht, vt = oracle.find_cross(Rc)
    pre = cc.copy()
    REF.ref_aggregate_cost_horizontal(P(pre), H, W, D)
    assert bits_equal(oracle.prefix_h(cc), pre)
    o = np.zeros_like(cc)
    REF.ref_cross_stereo_aggregation(P(pre.copy()), P(o), P(hl), P(ht), P(vl), P(vt), H, W, D)
    agg = oracle.cross_aggr(pre, hl, ht, vl, vt)
    assert bits_equal(agg, o)
    w = np.zeros((H, W), np.uint8)
    REF.ref_WTA(P(agg), P(w), H, W, D)
    assert bits_equal(oracle.wta(agg), w)
    w = np.zeros((H, W), np.uint8)
    REF.ref_WTA_NCC(P(agg), P(w), H, W, D)
    assert bits_equal(oracle.wta(agg, argmax=True), w)
    d2 = np.ascontiguousarray(np.roll(w, 3, axis=1))
    m = np.zeros((H, W), np.uint8)
    REF.ref_cross_check(P(w), P(d2), P(m), H, W)
    assert bits_equal(oracle.cross_check(w, d2), m)
    r1 = w.copy()
    REF.ref_disp_refinement(P(r1), P(hl), P(vl), H, W, D)
    assert bits_equal(oracle.disp_refinement(w, hl, vl, D, inplace=True), r1)


@pytest.mark.parametrize("rad", [1, 4])
def test_adaptive_weight(rad):
    H, W, D = 13, 17, 5
    L, R, Lc, Rc = pair(rad, H, W)
    pw = np.zeros(((2 * rad + 1) ** 2,), np.float32)
    REF.ref_calcProxWeight(P(pw), 36.0, rad)
    assert bits_equal(oracle.prox_weight(36.0, rad), pw)
    wl = np.zeros((H, W, pw.size), np.float32)
    REF.ref_computeWeights(P(wl), P(pw), P(Lc), 7.0, H, W, rad)
    assert bits_equal(oracle.compute_weights(pw, Lc, 7.0, rad), wl)
    wr = oracle.compute_weights(pw, Rc, 7.0, rad)
    cost = oracle.ad_color(Lc, Rc, D, 1, None, 1)
    o = np.zeros_like(cost)
    REF.ref_calcAWCostL2R(P(wl), P(wr), P(cost), P(o), H, W, D, rad)
    assert bits_equal(oracle.aw_l2r(wl, wr, cost, rad), o)
    a = cost.copy()
    REF.ref_calcAWCostR2L(P(wl), P(wr), P(a), H, W, D, rad)
    assert bits_equal(oracle.aw_r2l(wl, wr, cost, rad, inplace=True), a)


@pytest.mark.parametrize("c1,c2,ag,extra", [
    (1, 3, 3, {}), (1, 3, 1, {"box_rad": 4}), (1, 3, 2, {"aw_rad": 5}), (2, 3, 3, {"rank_rad": 3}),
    (4, 3, 3, {}), (5, 0, 1, {"box_rad": 2, "ncc_hrad": 3, "ncc_wrad": 3}), (3, 0, 3, {}), (4, 0, 2, {"aw_rad": 3}),
])
def test_whole_pipeline_vs_reference_composition(c1, c2, ag, extra):
    """The oracle's whole-pair pipeline against the reference's own functions
    composed in its driver's order (oracle.ref_pipeline, also the timed CPU
    baseline), colour and Lab images distinct from the gray ones; the box in place
    as the reference does it."""
    import rtstereo_gb300 as R
    H, W, D = 30, 64, 16
    L, Rr, Lc, Rc = pair(c1 * 100 + c2 * 10 + ag, H, W)
    Ll, Rl = R.rgb_to_lab(Lc), R.rgb_to_lab(Rc)
    p = oracle.params(D=D, cost1=c1, cost2=c2, aggr=ag, box_inplace=1, **extra)
    got = oracle.pipeline(p, L, Rr, Lc, Rc, Ll, Rl)[:3]
    want = oracle.ref_pipeline(p, L, Rr, Lc, Rc, Ll, Rl)
    for g, w in zip(got, want):
        assert bits_equal(g, w)
