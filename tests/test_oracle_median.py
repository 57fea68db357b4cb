"""The oracle's median pre-filter (OpenCV medianBlur as opencl/Main.cpp:342-343
applies it before findCross) against two independent statements of the same
filter: numpy over edge-padded windows, and scipy.ndimage.median_filter with
mode="nearest" (replicated borders).  OpenCV itself is not installed, so these
stand in for it; and the oracle pipeline's median option only changes the arms."""
import numpy as np
import pytest


def _numpy_median(img, k):
    r = k // 2
    a = img if img.ndim == 3 else img[:, :, None]
    pad = np.pad(a, ((r, r), (r, r), (0, 0)), mode="edge")
    win = np.lib.stride_tricks.sliding_window_view(pad, (k, k), axis=(0, 1))
    out = np.sort(win.reshape(win.shape[:3] + (k * k,)), axis=-1)[..., k * k // 2]
    return out.astype(np.uint8).reshape(img.shape)


@pytest.mark.parametrize("H,W", [(1, 1), (2, 3), (5, 40), (37, 23)])
@pytest.mark.parametrize("ch", [1, 3])
@pytest.mark.parametrize("k", [3, 5, 15])
def test_median_matches_numpy_and_scipy(oracle_mod, H, W, ch, k):
    rng = np.random.default_rng(H * 1000 + W * 10 + k)
    img = rng.integers(0, 256, (H, W) if ch == 1 else (H, W, 3), dtype=np.uint8)
    got = oracle_mod.median(img, k)
    assert np.array_equal(got, _numpy_median(img, k))
    nd = pytest.importorskip("scipy.ndimage")
    size = (k, k) if ch == 1 else (k, k, 1)
    assert np.array_equal(got, nd.median_filter(img, size=size, mode="nearest"))


def test_pipeline_median_changes_only_the_arms(oracle_mod):
    """With median_ksize the costs stay on the unfiltered images: feeding the
    filtered colour images as the colour input instead differs (AD uses colour)."""
    import rtstereo_gb300 as R
    O = oracle_mod
    H, W, D = 40, 64, 16
    L, Rr, _ = R.synth_pair(0x3ED1, W, H, D, 4, 0, 6.0, 3)
    rng = np.random.default_rng(5)
    Lc = np.ascontiguousarray(np.stack([L, rng.integers(0, 256, (H, W), dtype=np.uint8), L], -1))
    Rc = np.ascontiguousarray(np.stack([Rr, rng.integers(0, 256, (H, W), dtype=np.uint8), Rr], -1))
    p = O.params(D=D, median_ksize=3)
    with_med = O.pipeline(p, L, Rr, Lc, Rc)[0]
    plain = O.pipeline(O.params(D=D), L, Rr, Lc, Rc)[0]
    filtered_inputs = O.pipeline(O.params(D=D), L, Rr, O.median(Lc, 3), O.median(Rc, 3))[0]
    assert not np.array_equal(with_med, plain)
    assert not np.array_equal(with_med, filtered_inputs)
    # only the cross-based path reads the option
    pb = O.params(D=D, aggr=1)
    pb.median_ksize = 3
    assert np.array_equal(O.pipeline(pb, L, Rr, Lc, Rc)[0], O.pipeline(O.params(D=D, aggr=1), L, Rr, Lc, Rc)[0])
