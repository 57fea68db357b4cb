"""The headless driver rtstereo_gb300/rts_stereo (the reference driver's ten
arguments, seq/Main.cpp:50-61): argument handling on CPU, and its disparity
image against the oracle's left view scaled as seq/Main.cpp:258-274 on GPU."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "rtstereo_gb300", "rts_stereo")


def _driver():
    if not os.path.exists(DRIVER):
        from rtstereo_gb300 import build as B
        B.build()
    return DRIVER


def _write_pgm(path, img):
    with open(path, "wb") as f:
        f.write(b"P5\n%d %d\n255\n" % (img.shape[1], img.shape[0]))
        f.write(np.ascontiguousarray(img, np.uint8).tobytes())


def _read_png_gray(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, W = 8, b"", None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        assert zlib.crc32(kind + body) == struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if kind == b"IHDR":
            W, H, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 0
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(H, W + 1)
    assert (raw[:, 0] == 0).all()
    return raw[:, 1:]


def _scale_like_driver(disp, D, auto):
    # seq/Main.cpp:33 round() on the float product, then the 255 clamp
    if auto:
        coeff = np.float32(255) / np.float32(disp.max())
    else:
        coeff = np.float32({16: 16, 20: 8, 60: 4}[D])
    prod = disp.astype(np.float32) * coeff
    res = np.floor(prod.astype(np.float64) + 0.5)
    return np.minimum(res, 255).astype(np.uint8)


def test_usage_and_bad_images(tmp_path):
    exe = _driver()
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 255 and "Argument 10: Name of Dataset(Image)" in r.stdout
    r = subprocess.run([exe, str(tmp_path / "no.pgm"), str(tmp_path / "no.pgm")] + ["1"] * 7 + ["x"],
                       capture_output=True, text=True)
    assert r.returncode == 255 and "incorrect image data" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("args", [(16, 1, 3, 3, 0), (20, 3, 0, 1, 0), (24, 1, 3, 3, 1), (60, 2, 3, 3, 0)])
def test_driver_matches_oracle_left_view(tmp_path, oracle_mod, args):
    import rtstereo_gb300 as R
    D, c1, c2, ag, auto = args
    W, H = 96, 48
    L, Rr, _ = R.synth_pair(0xC0 + D, W, H, D, 5, 0, 2.0, 4)
    _write_pgm(tmp_path / "l.pgm", L)
    _write_pgm(tmp_path / "r.pgm", Rr)
    name = str(tmp_path / "set")
    r = subprocess.run([_driver(), str(tmp_path / "l.pgm"), str(tmp_path / "r.pgm"), str(D), str(c1), str(c2),
                        str(ag), str(auto), "10", "10", name], capture_output=True, text=True)
    assert r.returncode == 1, r.stdout
    got = _read_png_gray(f"{name}_{c1}_{c2}_{ag}_{auto}_10_10.png")
    Lc, Rc = R.gray_to_rgb(L), R.gray_to_rgb(Rr)
    O = oracle_mod
    dl, _, _, _ = O.pipeline(O.params(cost1=c1, cost2=c2, aggr=ag, D=D), L, Rr, Lc, Rc)
    assert np.array_equal(got, _scale_like_driver(dl, D, auto))


def _write_ppm(path, rgb):
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (rgb.shape[1], rgb.shape[0]))
        f.write(np.ascontiguousarray(rgb, np.uint8).tobytes())


@pytest.mark.gpu
def test_driver_colour_inputs(tmp_path, oracle_mod):
    """PPM inputs: the colour image feeds AD and the cross arms, its BT.601 luma
    (14-bit fixed point, as the driver converts) the gray costs."""
    import rtstereo_gb300 as R
    D, W, H = 16, 80, 40
    L, Rr, _ = R.synth_pair(0xC7, W, H, D, 4, 0, 2.0, 4)
    rng = np.random.default_rng(7)
    mk = lambda g: np.ascontiguousarray(np.stack([g, (g.astype(np.int32) * 3 // 4).astype(np.uint8),
                                                  np.clip(g.astype(np.int32) + rng.integers(-20, 21, g.shape), 0,
                                                          255).astype(np.uint8)], -1))
    Lc, Rc = mk(L), mk(Rr)
    _write_ppm(tmp_path / "l.ppm", Lc)
    _write_ppm(tmp_path / "r.ppm", Rc)
    name = str(tmp_path / "c")
    r = subprocess.run([_driver(), str(tmp_path / "l.ppm"), str(tmp_path / "r.ppm"), str(D), "1", "3", "3", "0",
                        "10", "10", name], capture_output=True, text=True)
    assert r.returncode == 1, r.stdout
    got = _read_png_gray(f"{name}_1_3_3_0_10_10.png")
    def luma(c):
        c = c.astype(np.uint32)
        return ((4899 * c[..., 0] + 9617 * c[..., 1] + 1868 * c[..., 2] + 8192) >> 14).astype(np.uint8)
    O = oracle_mod
    dl, _, _, _ = O.pipeline(O.params(D=D, right_view=0), luma(Lc), luma(Rc), Lc, Rc)
    assert np.array_equal(got, _scale_like_driver(dl, D, 0))
