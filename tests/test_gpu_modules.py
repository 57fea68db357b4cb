"""GPU parity of every module entry point (rts_<seq name>) against the C oracle,
through the C ABI.  The bar is bit-exact: every kernel keeps the reference's
per-entry arithmetic (integer costs exactly, float sums in the reference's
order without fused multiply-add, the C library's expf through host tables)."""
import ctypes as C

import numpy as np
import pytest

from conftest import bits_equal, smooth

pytestmark = pytest.mark.gpu

SIZES = [(7, 9, 1), (23, 37, 16), (31, 48, 32), (20, 300, 128), (5, 256, 256)]


def images(seed, H, W):
    rng = np.random.default_rng(seed)
    L = smooth(rng.integers(0, 256, (H, W), dtype=np.uint8))
    R = smooth(rng.integers(0, 256, (H, W), dtype=np.uint8))
    Lc = np.ascontiguousarray(np.stack([L, smooth(rng.integers(0, 256, (H, W), dtype=np.uint8)), L], -1))
    Rc = np.ascontiguousarray(np.stack([R, R, smooth(rng.integers(0, 256, (H, W), dtype=np.uint8))], -1))
    return L, R, Lc, Rc


@pytest.mark.parametrize("H,W,D", SIZES)
def test_ad(ctx, oracle_mod, H, W, D):
    O = oracle_mod
    L, R, Lc, Rc = images(1, H, W)
    assert bits_equal(ctx.pixelBasedL2R(L, R, D), O.ad_gray(L, R, D, O.L2R))
    assert bits_equal(ctx.pixelBasedR2L(L, R, D), O.ad_gray(L, R, D, O.R2L))
    for norm in (0, 1):
        for tr in (None, 24.0, 7.5):
            assert bits_equal(ctx.pixelBasedCostL2R_Color(Lc, Rc, D, norm, tr), O.ad_color(Lc, Rc, D, O.L2R, tr, norm))
            assert bits_equal(ctx.pixelBasedR2L_Color(Lc, Rc, D, norm, tr), O.ad_color(Lc, Rc, D, O.R2L, tr, norm))
    if min(H, W) > 2:
        Lf, Rf = ctx.convolveImage(L), ctx.convolveImage(R)
        assert bits_equal(Lf, O.convolve(L, O.LOG5x5, 2, 2))
        assert bits_equal(ctx.pixelBasedCostL2R_Float(Lf, Rf, D), O.ad_float(Lf, Rf, D, O.L2R))
        assert bits_equal(ctx.pixelBasedCostR2L_Float(Lf, Rf, D), O.ad_float(Lf, Rf, D, O.R2L))


@pytest.mark.parametrize("H,W,D", SIZES)
@pytest.mark.parametrize("hr,wr", [(4, 3), (1, 1), (5, 7)])
def test_census_hamming(ctx, oracle_mod, H, W, D, hr, wr):
    O = oracle_mod
    if hr >= H or wr >= W:
        pytest.skip("window larger than the image")
    L, R, _, _ = images(2, H, W)
    bl, br = ctx.calcCensusTrans(L, hr, wr), ctx.calcCensusTrans(R, hr, wr)
    assert bits_equal(bl, O.census(L, hr, wr)) and bits_equal(br, O.census(R, hr, wr))
    assert bits_equal(ctx.calcHammingDist(bl, br, D, hr, wr), O.hamming(bl, br, D, hr, wr))


@pytest.mark.parametrize("H,W,D", SIZES[:4])
def test_rank_ncc(ctx, oracle_mod, H, W, D):
    O = oracle_mod
    L, R, _, _ = images(3, H, W)
    for m in (1, 3, 7):
        if m < min(H, W):
            assert bits_equal(ctx.calculateRankFilt(L, m), O.rank(L, m))
    for r in (1, 3):
        if r < H and r + D <= W:
            assert bits_equal(ctx.calcNCCDispL2R(L, R, D, r, r, fill=-7.0), O.ncc(L, R, D, r, r, fill=-7.0))
    if D + 1 <= W and H > 1:
        flat = np.full((H, W), 9, np.uint8)  # zero denominators: cells stay unwritten
        assert bits_equal(ctx.calcNCCDispL2R(flat, R, D, 1, 1, fill=-7.0), O.ncc(flat, R, D, 1, 1, fill=-7.0))


@pytest.mark.parametrize("H,W,D", SIZES)
def test_combine_box_cross_wta(ctx, oracle_mod, H, W, D):
    O = oracle_mod
    L, R, Lc, Rc = images(4, H, W)
    c1 = O.ad_color(Lc, Rc, D, O.L2R, 24.0, 0)
    c2 = O.ad_gray(L, R, D, O.L2R)
    for l1, l2 in ((10.0, 10.0), (7.0, 30.0)):
        assert bits_equal(ctx.combineCost(c1, c2, l1, l2), O.combine(c1, c2, l1, l2))
    # non-integer inputs take the device expf: within 2 ulp-ish of the C library
    f1 = (c1 * 0.37).astype(np.float32)
    got, want = ctx.combineCost(f1, c2, 10.0, 10.0), O.combine(f1, c2, 10.0, 10.0)
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-6)
    cc = O.combine(c1, c2, 10.0, 10.0)
    for r in (1, 4):
        if r < min(H, W):
            assert bits_equal(ctx.boxAggregate(cc, r), O.box(cc, r))
    hl, vl = ctx.findCross(Lc)
    ht, vt = ctx.findCross(Rc)
    ohl, ovl = O.find_cross(Lc)
    assert bits_equal(hl, ohl) and bits_equal(vl, ovl)
    pre = ctx.aggregate_cost_horizontal(cc)
    assert bits_equal(pre, O.prefix_h(cc))
    agg = ctx.cross_stereo_aggregation(pre, hl, ht, vl, vt)
    oagg = O.cross_aggr(pre, hl, ht, vl, vt)
    assert bits_equal(agg, oagg)
    assert bits_equal(ctx.WTA(agg), O.wta(agg))
    assert bits_equal(ctx.WTA_NCC(agg), O.wta(agg, argmax=True))
    d = O.wta(agg)
    d2 = np.ascontiguousarray(np.roll(d, 3, axis=1))
    assert bits_equal(ctx.cross_check(d, d2), O.cross_check(d, d2))
    assert bits_equal(ctx.disp_refinement(d, hl, vl, D), O.disp_refinement(d, hl, vl, D))


def test_wta_carry_known_answer(ctx, oracle_mod):
    # seq/WTA.cpp:12: the winner is not reset per pixel.  Pixel 1 has its
    # minimum at d=0, so it keeps pixel 0's winner 3.
    cost = np.array([[[5, 5, 5, 1], [0, 5, 5, 5], [4, 4, 4, 4], [9, 2, 2, 1]]], np.float32)
    assert ctx.WTA(cost).tolist() == [[3, 3, 3, 3]]
    assert oracle_mod.wta(cost).tolist() == [[3, 3, 3, 3]]
    # the carry crosses rows and empty rows, and starts at 0
    rng = np.random.default_rng(5)
    H, W, D = 70, 45, 8
    cost = rng.integers(0, 3, (H, W, D)).astype(np.float32)
    cost[:, :, 0] = 0  # most pixels have no strictly better d >= 1
    cost[10:40] = 1
    cost[10:40, :, 0] = 0
    cost[50, 7, 5] = -1
    assert bits_equal(ctx.WTA(cost), oracle_mod.wta(cost))
    assert bits_equal(ctx.WTA_NCC(cost), oracle_mod.wta(cost, argmax=True))


@pytest.mark.parametrize("rad", [1, 3, 8])
def test_adaptive_weight(ctx, oracle_mod, rad):
    O = oracle_mod
    H, W, D = 21, 33, 8
    _, _, Lc, Rc = images(6, H, W)
    pw = ctx.calcProxWeight(36.0, rad)
    assert bits_equal(pw, O.prox_weight(36.0, rad))
    wl = ctx.computeWeights(pw, Lc, 7.0, rad)
    wr = ctx.computeWeights(pw, Rc, 7.0, rad)
    assert bits_equal(wl, O.compute_weights(pw, Lc, 7.0, rad))
    cost = O.ad_color(Lc, Rc, D, O.L2R, None, 1)
    assert bits_equal(ctx.calcAWCostL2R(wl, wr, cost, rad), O.aw_l2r(wl, wr, cost, rad))
    assert bits_equal(ctx.calcAWCostR2L(wl, wr, cost, rad), O.aw_r2l(wl, wr, cost, rad))


def test_device_pointers_and_stream(ctx, oracle_mod):
    """DEVICE-mode call on torch buffers and torch's stream."""
    torch = pytest.importorskip("torch")
    import rtstereo_gb300 as R
    O = oracle_mod
    H, W, D = 40, 64, 16
    L, Rr, Lc, Rc = images(7, H, W)
    dl, dr = torch.from_numpy(Lc).cuda(), torch.from_numpy(Rc).cuda()
    out = torch.empty((H, W, D), dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()  # a real stream handle (the legacy default stream is handle 0)
    s.wait_stream(torch.cuda.current_stream())
    ctx.set_stream(s.cuda_stream)
    try:
        ctx.call("pixelBasedCostL2R_Color_trunc", R.DEVICE, dl, dr, out, D, H, W, C.c_float(24.0), 0)
        s.synchronize()
    finally:
        ctx.set_stream(None)
    assert bits_equal(out.cpu().numpy(), O.ad_color(Lc, Rc, D, O.L2R, 24.0, 0))


def test_invalid_arguments_report_status(ctx):
    import rtstereo_gb300 as R
    L = np.zeros((4, 4), np.uint8)
    with pytest.raises(R.RtsError) as e:
        ctx.pixelBasedL2R(L, L, 5)  # D > W
    assert e.value.status == 1
    with pytest.raises(R.RtsError):
        ctx.calcCensusTrans(L, 4, 3)  # window larger than the image
