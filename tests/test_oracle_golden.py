"""The C oracle against the committed fixtures made by the reference's own seq/
code (tests/golden/make_golden.py).  CPU only; this pins the oracle on every
machine, including the ones where the reference tree is absent."""
import numpy as np
import pytest

from conftest import bits_equal

def test_matching_costs(golden, oracle_mod):
    O = oracle_mod
    L, R, Lc, Rc = golden["img/L"], golden["img/R"], golden["img/Lc"], golden["img/Rc"]
    D = golden["pixelBasedL2R"].shape[2]
    assert bits_equal(O.ad_gray(L, R, D, O.L2R), golden["pixelBasedL2R"])
    assert bits_equal(O.ad_gray(L, R, D, O.R2L), golden["pixelBasedR2L"])
    for n in (0, 1):
        assert bits_equal(O.ad_color(Lc, Rc, D, O.L2R, None, n), golden[f"L2R_Color/n{n}"])
        assert bits_equal(O.ad_color(Lc, Rc, D, O.R2L, None, n), golden[f"R2L_Color/n{n}"])
        assert bits_equal(O.ad_color(Lc, Rc, D, O.L2R, 24.0, n), golden[f"L2R_Color_trunc24/n{n}"])
        assert bits_equal(O.ad_color(Lc, Rc, D, O.R2L, 24.0, n), golden[f"R2L_Color_trunc24/n{n}"])
    Lf = O.convolve(L, O.LOG5x5, 2, 2)
    Rf = O.convolve(R, O.LOG5x5, 2, 2)
    assert bits_equal(Lf, golden["convolveImage/L"]) and bits_equal(Rf, golden["convolveImage/R"])
    assert bits_equal(O.ad_float(Lf, Rf, D, O.L2R), golden["pixelBasedCostL2R_Float"])
    assert bits_equal(O.ad_float(Lf, Rf, D, O.R2L), golden["pixelBasedCostR2L_Float"])


@pytest.mark.parametrize("hr,wr", [(4, 3), (2, 5)])
def test_census_hamming(golden, oracle_mod, hr, wr):
    O = oracle_mod
    L, R = golden["img/L"], golden["img/R"]
    D = golden["pixelBasedL2R"].shape[2]
    bl, br = O.census(L, hr, wr), O.census(R, hr, wr)
    assert bits_equal(bl, golden[f"census{hr}x{wr}/L"]) and bits_equal(br, golden[f"census{hr}x{wr}/R"])
    assert bits_equal(O.hamming(bl, br, D, hr, wr), golden[f"hamming{hr}x{wr}"])


def test_rank_ncc(golden, oracle_mod):
    O = oracle_mod
    L, R = golden["img/L"], golden["img/R"]
    D = golden["pixelBasedL2R"].shape[2]
    for m in (1, 3, 7):
        assert bits_equal(O.rank(L, m), golden[f"rank{m}"])
    for r in (1, 3):
        assert bits_equal(O.ncc(L, R, D, r, r, fill=-7.0), golden[f"ncc{r}x{r}"])
    flat = np.full(L.shape, 9, np.uint8)
    assert bits_equal(O.ncc(flat, R, D, 1, 1, fill=-7.0), golden["ncc_flat1x1"])


def test_combine_box_cross_wta(golden, oracle_mod):
    O = oracle_mod
    c1, c2 = golden["L2R_Color_trunc24/n0"], golden["hamming4x3"]
    assert bits_equal(O.combine(c1, c2, 10.0, 10.0), golden["combine/10_10"])
    assert bits_equal(O.combine(c1, c2, 7.0, 30.0), golden["combine/7_30"])
    cc = golden["combine/10_10"]
    for r in (1, 4):
        assert bits_equal(O.box(cc, r, inplace=True), golden[f"box_inplace{r}"])
    hl, vl = O.find_cross(golden["img/Lc"])
    ht, vt = O.find_cross(golden["img/Rc"])
    assert bits_equal(hl, golden["findCross/Lh"]) and bits_equal(vl, golden["findCross/Lv"])
    assert bits_equal(ht, golden["findCross/Rh"]) and bits_equal(vt, golden["findCross/Rv"])
    pre = O.prefix_h(cc)
    assert bits_equal(pre, golden["prefix"])
    agg = O.cross_aggr(pre, hl, ht, vl, vt)
    assert bits_equal(agg, golden["cross"])
    assert bits_equal(O.wta(agg), golden["WTA/cross"])
    assert bits_equal(O.wta(golden["WTA/ties_in"]), golden["WTA/ties"])
    assert bits_equal(O.wta(golden["WTA/ties_in"], argmax=True), golden["WTA_NCC/ties"])
    assert bits_equal(O.cross_check(golden["WTA/cross"], golden["cross_check/tar"]), golden["cross_check"])


@pytest.mark.parametrize("rad", [3, 7])
def test_adaptive_weight(golden, oracle_mod, rad):
    O = oracle_mod
    pw = O.prox_weight(36.0, rad)
    assert bits_equal(pw, golden[f"aw{rad}/prox"])
    wl = O.compute_weights(pw, golden["aw/labL"], 7.0, rad)
    wr = O.compute_weights(pw, golden["aw/labR"], 7.0, rad)
    if rad == 3:
        assert bits_equal(wl, golden["aw3/wL"])
        assert bits_equal(O.aw_r2l(wl, wr, golden["aw/cost"], rad, inplace=True), golden["aw3/r2l_inplace"])
    assert bits_equal(O.aw_l2r(wl, wr, golden["aw/cost"], rad), golden[f"aw{rad}/l2r"])


@pytest.mark.parametrize("name,c1,c2,ag", [("pipe_ad_census_cross", 1, 3, 3), ("pipe_ad_census_box", 1, 3, 1),
                                           ("pipe_rank_census_aw", 2, 3, 2)])
def test_pipeline(golden, oracle_mod, name, c1, c2, ag):
    O = oracle_mod
    import rtstereo_gb300 as R
    L, Rg = golden[f"{name}/L"], golden[f"{name}/R"]
    H, W = L.shape
    D = {"pipe_ad_census_cross": 16, "pipe_ad_census_box": 8, "pipe_rank_census_aw": 6}[name]
    p = O.params(cost1=c1, cost2=c2, aggr=ag, D=D, box_rad=1, rank_rad=7, box_inplace=1,
                 aw_rad=16 if min(H, W) > 16 else 5)
    rgb = lambda a: np.ascontiguousarray(np.repeat(a[:, :, None], 3, axis=2))
    lab = (R.rgb_to_lab(rgb(L)), R.rgb_to_lab(rgb(Rg))) if ag == 2 else (None, None)
    dl, dr, mk, _ = O.pipeline(p, L, Rg, rgb(L), rgb(Rg), *lab)
    assert bits_equal(dl, golden[f"{name}/disp_left"])
    assert bits_equal(dr, golden[f"{name}/disp_right"])
    assert bits_equal(mk, golden[f"{name}/mask"])
