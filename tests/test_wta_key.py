"""The WTA order key of the device arg-min kernels (`wta_key` in
rtstereo_gb300/csrc/rts_common.cuh, used by k_wta_local, k_box_best,
k_box_best_dp and the FP16 box kernel's right-view minima), restated in numpy:
the least {key, d} over d must be the reference's sequential winner
(seq/WTA.cpp:10-39) -- the first strict minimum (maximum for WTA_NCC) in
increasing d, a NaN never winning, a NaN at d = 0 blocking every other d,
-0 == +0 -- and "found" (some d >= 1 won) must be winner != 0."""
import numpy as np
import pytest


def wta_key(v, d, argmax):
    """The device key of float32 cost v at disparity d (uint32)."""
    v = np.float32(v)
    if v != v:
        return 0 if d == 0 else 0xFFFFFFFF
    u = int((v + np.float32(0.0)).view(np.uint32))  # -0 -> +0
    u = (~u & 0xFFFFFFFF) if u & 0x80000000 else (u | 0x80000000)
    return (~u & 0xFFFFFFFF) if argmax else u


def ref_winner(c, argmax):
    """seq/WTA.cpp: best = c[0], then d = 1.. replaces it on a strict improvement."""
    best, win, found = c[0], 0, False
    for d in range(1, len(c)):
        v = c[d]
        if (v > best) if argmax else (v < best):
            best, win, found = v, d, True
    return win, found


def key_winner(c, argmax):
    return min((wta_key(v, d, argmax), d) for d, v in enumerate(c))[1]


SPECIAL = np.array([np.nan, -np.inf, -1.0, -0.0, 0.0, 0.5, 1.0, np.inf], np.float32)


@pytest.mark.parametrize("argmax", [0, 1])
@pytest.mark.parametrize("D", [1, 2, 7, 32, 33, 128])
def test_key_order_is_the_reference_winner(D, argmax):
    rng = np.random.default_rng(1000 * D + argmax)
    for case in range(300):
        if case % 3 == 0:
            c = SPECIAL[rng.integers(len(SPECIAL), size=D)]  # ties, signed zeros, infinities, NaNs
        elif case % 3 == 1:
            c = rng.integers(0, 4, size=D).astype(np.float32)  # many ties
        else:
            c = rng.standard_normal(D).astype(np.float32)
            c[rng.random(D) < 0.1] = np.nan
        win, found = ref_winner(c, argmax)
        got = key_winner(c, argmax)
        assert got == win, (c.tolist(), argmax)
        assert (got != 0) == found


def test_nan_at_zero_blocks_and_no_number_takes_its_key():
    c = np.array([np.nan, -5.0, -np.inf], np.float32)
    assert ref_winner(c, 0) == (0, False) and key_winner(c, 0) == 0
    assert ref_winner(c, 1) == (0, False) and key_winner(c, 1) == 0
    # no number has the key of a NaN at d = 0 (0) or after it (all ones)
    for v in SPECIAL[1:]:
        for argmax in (0, 1):
            assert 0 < wta_key(v, 3, argmax) < 0xFFFFFFFF
