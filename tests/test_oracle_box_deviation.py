"""How far the GPU contract's out-of-place forms (every window reads the
unmodified input) are from the reference's literal in-place recurrences, where
later windows read cells already overwritten: the box aggregation
(seq/ConstBlockAggregation.cpp:27,31), calcAWCostR2L and disp_refinement.  Both
forms come from the oracle, the in-place ones pinned to the reference
elsewhere.  CPU only; run with -s to print the figures."""
import numpy as np
import pytest


@pytest.mark.parametrize("rad", [1, 4])
def test_box_inplace_deviation(oracle_mod, rad):
    import rtstereo_gb300 as R
    O = oracle_mod
    # the 384x288, D=16 random-dot pair (6 rectangles, noise 2), gray read as colour
    L, Rr, _ = R.synth_pair(0xC0, 384, 288, 16, 6, 0, 2.0, 4)
    rgb = lambda a: np.ascontiguousarray(np.repeat(a[:, :, None], 3, axis=2))
    out = {}
    for inplace in (0, 1):
        p = O.params(D=16, cost1=1, cost2=3, aggr=1, box_rad=rad, box_inplace=inplace)
        out[inplace] = O.pipeline(p, L, Rr, rgb(L), rgb(Rr), want_cost=True)
    oop, inp = out[0], out[1]
    diff = np.abs(oop[3] - inp[3])
    equal_l = float(np.mean(oop[0] == inp[0]))
    equal_m = float(np.mean(oop[2] == inp[2]))
    print(f"\nbox r={rad}: left disparities equal {100 * equal_l:.2f} %, masks equal {100 * equal_m:.2f} %, "
          f"largest cost difference {diff.max() / np.abs(inp[3]).max():.3g} of the largest cost, "
          f"mean {diff.mean() / np.abs(inp[3]).mean():.3g} of the mean")
    assert diff.max() > 0  # the recurrence does change the volume
    assert equal_l > 0.98 and equal_m > 0.98  # ... and few winners


def test_aw_r2l_and_refinement_inplace_deviation(oracle_mod):
    """The same for the other two in-place functions: calcAWCostR2L
    (seq/AdaptiveWeightAggregation.cpp:147) and disp_refinement
    (seq/CrossBasedAggregation.cpp:208)."""
    import rtstereo_gb300 as R
    O = oracle_mod
    W, H, D, rad = 96, 64, 16, 4
    L, Rr, _ = R.synth_pair(0xC1, W, H, D, 4, 1, 2.0, 4)
    rgb = lambda a: np.ascontiguousarray(np.repeat(a[:, :, None], 3, axis=2))
    Lc, Rc = rgb(L), rgb(Rr)
    pw = O.prox_weight(36.0, rad)
    wl = O.compute_weights(pw, R.rgb_to_lab(Lc), 7.0, rad)
    wr = O.compute_weights(pw, R.rgb_to_lab(Rc), 7.0, rad)
    cost = O.ad_color(Rc, Lc, D, O.R2L, None, 0)
    a, b = O.aw_r2l(wr, wl, cost, rad), O.aw_r2l(wr, wl, cost, rad, inplace=True)
    d_aw = float(np.abs(a - b).max() / np.abs(b).max())
    eq_aw = float(np.mean(O.wta(a) == O.wta(b)))
    # refinement of the cross-based left disparity of the 384x288 pair
    L, Rr, _ = R.synth_pair(0xC0, 384, 288, 16, 6, 0, 2.0, 4)
    disp = O.pipeline(O.params(D=16), L, Rr, rgb(L), rgb(Rr))[0]
    horz, vert = O.find_cross(rgb(L))
    ra, rb = O.disp_refinement(disp, horz, vert, 16), O.disp_refinement(disp, horz, vert, 16, inplace=True)
    eq_ref = float(np.mean(ra == rb))
    print(f"\ncalcAWCostR2L r={rad}: largest cost difference {d_aw:.3g} of the largest cost, winners equal "
          f"{100 * eq_aw:.2f} %; disp_refinement: {100 * eq_ref:.2f} % of the disparities equal")
    assert d_aw > 0 and eq_aw > 0.9
    assert eq_ref < 1.0 and eq_ref > 0.5
