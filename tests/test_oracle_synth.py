"""The oracle's host-side helpers (no GPU): its input generator is the
library's, bit for bit (the CPU reference arm makes its inputs with it so that
it never loads the library); its results do not depend on the number of host
threads; its row-range adaptive-weight functions equal the whole-image ones."""
import numpy as np
import pytest


@pytest.mark.parametrize("seed,W,H,D,rects,planes,sigma", [(0xC0, 384, 288, 16, 6, 0, 2.0),
                                                             (0xC1, 640, 480, 64, 12, 1, 2.0),
                                                             (0xC2, 333, 97, 128, 24, 2, 3.0),
                                                             (7, 5, 3, 2, 1, 1, 0.0)])
def test_oracle_generator_is_the_library_generator(oracle_mod, seed, W, H, D, rects, planes, sigma):
    import rtstereo_gb300 as R
    a = oracle_mod.synth_pair(seed, W, H, D, rects, planes, sigma, min(4, D - 1))
    b = R.synth_pair(seed, W, H, D, rects, planes, sigma, min(4, D - 1))
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    rgb = oracle_mod.gray_to_rgb(a[0])
    assert np.array_equal(rgb, R.gray_to_rgb(a[0]))
    colour = np.random.default_rng(seed).integers(0, 256, (H, W, 3), dtype=np.uint8)
    assert np.array_equal(oracle_mod.rgb_to_lab(colour), R.rgb_to_lab(colour))
    assert np.array_equal(oracle_mod.rgb_to_lab(rgb), R.rgb_to_lab(rgb))


def test_oracle_results_do_not_depend_on_threads(oracle_mod):
    O = oracle_mod
    L, Rr, _ = O.synth_pair(0x51, 96, 40, 24, 4, 1, 2.0, 4)
    Lc, Rc = O.gray_to_rgb(L), O.gray_to_rgb(Rr)
    Ll, Rl = O.rgb_to_lab(Lc), O.rgb_to_lab(Rc)
    runs = []
    for n in (1, 0):
        O.set_threads(n)
        out = []
        for kw in (dict(aggr=3), dict(aggr=1, box_rad=2), dict(aggr=2, aw_rad=4), dict(cost1=5, cost2=0, aggr=1),
                   dict(cost1=2, cost2=3, aggr=3, rank_rad=3, median_ksize=3)):
            out.append(O.pipeline(O.params(D=24, **kw), L, Rr, Lc, Rc, Ll, Rl, want_cost=True))
        runs.append(out)
    O.set_threads(0)
    for a, b in zip(*runs):
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))


def test_oracle_adaptive_weight_rows_equal_whole_image(oracle_mod):
    O = oracle_mod
    L, Rr, _ = O.synth_pair(0x52, 70, 36, 16, 4, 1, 2.0, 4)
    Lc, Rc = O.gray_to_rgb(L), O.gray_to_rgb(Rr)
    Ll, Rl = O.rgb_to_lab(Lc), O.rgb_to_lab(Rc)
    p = O.params(D=16, aggr=2, aw_rad=5, right_view=0)
    vol = O.view_cost(p, L, Rr, Lc, Rc)
    pw = O.prox_weight(p.aw_gamma_p, p.aw_rad)
    full = O.aw_l2r(O.compute_weights(pw, Ll, p.aw_gamma_s, p.aw_rad), O.compute_weights(pw, Rl, p.aw_gamma_s, p.aw_rad),
                    vol, p.aw_rad)
    rows = [0, 3, 17, 35]
    part = O.aw_l2r_rows(Ll, Rl, vol, rows, p.aw_rad, p.aw_gamma_s, p.aw_gamma_p)
    assert np.array_equal(part.view(np.uint32), full[rows].view(np.uint32))
    # and the pipeline's own final volume
    whole = O.pipeline(p, L, Rr, Lc, Rc, Ll, Rl, want_cost=True)[3]
    assert np.array_equal(whole.view(np.uint32), full.view(np.uint32))
