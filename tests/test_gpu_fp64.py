"""Float costs against FP64 restatements of the same formulas (the oracle's
orc64_* functions): the plain form, bit-exact to the reference's fp32
arithmetic, stays within 1e-4 of FP64 relative to the volume's largest
magnitude; the FP16 form's adaptive-weight volume (FP16 storage of the cost
volume, fp32 accumulation) is reported against FP64 with its WTA agreement.
Run with -s to see the measured errors."""
import numpy as np
import pytest

from conftest import smooth

pytestmark = pytest.mark.gpu


def rel_err(got, want):
    got = np.asarray(got, np.float64)
    return float(np.abs(got - want).max() / max(np.abs(want).max(), 1e-30))


def images(seed, H, W):
    rng = np.random.default_rng(seed)
    L = smooth(rng.integers(0, 256, (H, W), dtype=np.uint8))
    R = np.roll(L, -3, axis=1)
    R = np.clip(R.astype(np.int16) + rng.integers(-4, 5, (H, W)), 0, 255).astype(np.uint8)
    return L, R


def test_plain_module_costs_vs_fp64(ctx, oracle_mod):
    O = oracle_mod
    H, W, D = 40, 96, 24
    L, Rr = images(11, H, W)
    e_log = rel_err(ctx.convolveImage(L), O.f64_convolve(L, O.LOG5x5, 2, 2))
    e_ncc = rel_err(ctx.calcNCCDispL2R(L, Rr, D, 3, 3), O.f64_ncc(L, Rr, D, 3, 3))
    Lc, Rc = np.repeat(L[:, :, None], 3, 2).copy(), np.repeat(Rr[:, :, None], 3, 2).copy()
    c1 = O.ad_color(Lc, Rc, D)
    c2 = O.hamming(O.census(L), O.census(Rr), D)
    e_comb = rel_err(ctx.combineCost(c1, c2, 10.0, 10.0), O.f64_combine(c1, c2, 10.0, 10.0))
    print(f"\nplain vs FP64 (relative to max |FP64|): LoG {e_log:.2e}, NCC {e_ncc:.2e}, combine {e_comb:.2e}")
    assert max(e_log, e_ncc, e_comb) < 1e-4


def test_adaptive_weight_forms_vs_fp64(ctx, oracle_mod):
    import rtstereo_gb300 as R
    O = oracle_mod
    H, W, D, rad = 48, 96, 24, 16
    L, Rr = images(12, H, W)
    Lc, Rc = R.gray_to_rgb(L), R.gray_to_rgb(Rr)
    Ll, Rl = R.rgb_to_lab(Lc), R.rgb_to_lab(Rc)
    # FP64: the same AD and census terms combined and aggregated in double precision
    c1 = O.ad_color(Lc, Rc, D)
    c2 = O.hamming(O.census(L), O.census(Rr), D)
    want = O.f64_aw_l2r_pre(Ll, Rl, O.f64_combine(c1, c2, 10.0, 10.0), rad, 7.0, 36.0)
    got = {}
    for prec in (R.PREC_F32, R.PREC_F16):
        p = R.params(cost1=1, cost2=3, aggr=2, disp_range=D, aw_rad=rad, right_view=0, precision=prec)
        got[prec] = ctx.pipeline(p, L, Rr, Lc, Rc, Ll, Rl, want_cost=True)
    e32 = rel_err(got[R.PREC_F32][3], want)
    e16 = rel_err(got[R.PREC_F16][3], want)
    a16 = float((got[R.PREC_F16][0] == got[R.PREC_F32][0]).mean())
    print(f"\nadaptive weights vs FP64 (relative to max |FP64|): plain {e32:.2e}, FP16 form {e16:.2e}; "
          f"FP16 WTA agreement with plain {100 * a16:.3f} %")
    assert e32 < 1e-4
    assert e16 < 2e-3
    assert a16 > 0.99
