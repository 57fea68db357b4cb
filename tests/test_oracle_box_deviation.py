"""How far the GPU contract's box aggregation (out of place: every window reads
the unaggregated volume) is from the reference's literal in-place recurrence
(seq/ConstBlockAggregation.cpp:27,31: later windows read cells already
overwritten).  Both forms come from the oracle, the in-place one pinned to the
reference elsewhere.  CPU only; run with -s to print the figures."""
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
