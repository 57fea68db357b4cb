"""CPU oracle for the rtstereo per-frame stereo pipeline -- TEST INFRASTRUCTURE ONLY.

Two libraries sit behind this module:

* ``librts_oracle.so`` -- the plain-C restatement in ``rts_oracle.c`` (always
  built by ``make -C oracle``), the checker the GPU tests compare against;
* ``_ref/libseqref.so`` -- the reference's own ``seq/*.cpp`` compiled from its
  sources (built only where the reference tree is present), used to pin the
  restatement and to make ``tests/golden``.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this package.  Arrays are numpy, in the reference's layouts (cost
volume ``[H][W][D]`` float32, images ``[H][W]`` / ``[H][W][3]`` uint8).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librts_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libseqref.so")

L2R, R2L = 1, -1

_p = C.c_void_p
_i = C.c_int
_f = C.c_float
_d = C.c_double
_l = C.c_long

# name -> argtypes, for librts_oracle.so
_ORACLE_SIGS = {
    "orc_ad_gray": [_p, _p, _p, _i, _i, _i, _i],
    "orc_ad_float": [_p, _p, _p, _i, _i, _i, _i],
    "orc_ad_color": [_p, _p, _p, _i, _i, _i, _i, _i, _f, _i],
    "orc_census": [_p, _p, _i, _i, _i, _i],
    "orc_hamming": [_p, _p, _p, _i, _i, _i, _i, _i],
    "orc_rank": [_p, _p, _i, _i, _i],
    "orc_convolve": [_p, _p, _p, _i, _i, _i, _i],
    "orc_ncc": [_p, _p, _p, _i, _i, _i, _i, _i],
    "orc_combine": [_p, _p, _f, _f, _i, _i, _i],
    "orc_box_inplace": [_p, _i, _i, _i, _i],
    "orc_box": [_p, _p, _i, _i, _i, _i],
    "orc_find_cross": [_p, _p, _p, _i, _i, _i, _i],
    "orc_median": [_p, _p, _i, _i, _i, _i],
    "orc_prefix_h": [_p, _i, _i, _i],
    "orc_cross_aggr": [_p, _p, _p, _p, _p, _p, _i, _i, _i],
    "orc_prox_weight": [_p, _f, _i],
    "orc_compute_weights": [_p, _p, _p, _f, _i, _i, _i],
    "orc_aw_l2r": [_p, _p, _p, _p, _i, _i, _i, _i],
    "orc_aw_r2l": [_p, _p, _p, _i, _i, _i, _i],
    "orc_aw_r2l_oop": [_p, _p, _p, _p, _i, _i, _i, _i],
    "orc_wta": [_p, _p, _i, _i, _i, _i],
    "orc_cross_check": [_p, _p, _p, _i, _i],
    "orc_disp_refinement": [_p, _p, _p, _i, _i, _i],
    "orc_disp_refinement_oop": [_p, _p, _p, _p, _i, _i, _i],
    "orc64_combine": [_p, _p, _d, _d, _l, _p],
    "orc64_aw_l2r": [_p, _p, _p, _p, _i, _i, _i, _i, _d, _d],
    "orc64_aw_l2r_pre": [_p, _p, _p, _p, _i, _i, _i, _i, _d, _d],
    "orc64_ncc": [_p, _p, _p, _i, _i, _i, _i, _i],
    "orc64_convolve": [_p, _p, _p, _i, _i, _i, _i],
    "orc_pipeline": [_p, _i, _i, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p],
    "orc_compute_weights_rows": [_p, _p, _p, _f, _i, _i, _i, _i, _i],
    "orc_aw_l2r_rows": [_p, _p, _p, _p, _i, _i, _i, _i, _i, _i],
    "orc_view_cost": [_p, _i, _i, _p, _p, _p, _p, _p],
    "orc_set_threads": [_i],
    "orc_threads": [],
    "orc_synth_pair": [C.c_uint64, _i, _i, _i, _i, _i, _f, _i, _p, _p, _p],
    "orc_gray_to_rgb": [_p, _p, _i, _i],
    "orc_rgb_to_lab": [_p, _p, _i, _i],
}
_INT_RESULT = ("orc_pipeline", "orc64_aw_l2r_pre", "orc_view_cost", "orc_threads", "orc_synth_pair")


class OrcParams(C.Structure):
    """Mirror of ``orc_params`` in rts_oracle.h."""

    _fields_ = [
        ("cost1", _i), ("cost2", _i), ("aggr", _i),
        ("lambda1", _f), ("lambda2", _f),
        ("D", _i),
        ("census_hrad", _i), ("census_wrad", _i),
        ("rank_rad", _i),
        ("ncc_hrad", _i), ("ncc_wrad", _i),
        ("box_rad", _i),
        ("aw_rad", _i),
        ("aw_gamma_s", _f), ("aw_gamma_p", _f),
        ("cross_L", _i), ("cross_tau", _i),
        ("ad_trunc", _f),
        ("right_view", _i),
        ("box_inplace", _i),
        ("median_ksize", _i),
    ]


def build(force: bool = False) -> None:
    """Compile the restatement with gcc (same flags as oracle/Makefile): with
    OpenMP where the compiler has it (row loops on all host threads), else
    serial; the results are the same either way."""
    src = os.path.join(HERE, "rts_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "rts_oracle.h"))):
        tmp = LIB_PATH + ".tmp"
        base = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp, src, "-lm"]
        if subprocess.run(base[:1] + ["-fopenmp"] + base[1:], capture_output=True).returncode != 0:
            subprocess.run(base, check=True, capture_output=True)
        os.replace(tmp, LIB_PATH)


def _bind(lib, sigs):
    for name, args in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _i if name in _INT_RESULT else None
    return lib


_LIB = None
_REF = None


def lib():
    global _LIB
    if _LIB is None:
        build()
        _LIB = _bind(C.CDLL(LIB_PATH), _ORACLE_SIGS)
    return _LIB


def have_reference() -> bool:
    return os.path.exists(REF_PATH)


def reflib():
    """The reference's own seq/ code (oracle/_ref), or None when not built."""
    global _REF
    if _REF is None and have_reference():
        r = C.CDLL(REF_PATH)
        for name in ["ref_pixelBasedL2R", "ref_pixelBasedR2L", "ref_pixelBasedCostL2R_Float",
                     "ref_pixelBasedCostR2L_Float", "ref_pixelBasedCostL2R_Color",
                     "ref_pixelBasedR2L_Color", "ref_calcCensusTrans", "ref_calcHammingDist",
                     "ref_calculateRankFilt", "ref_convolveImage", "ref_calcNCCDispL2R",
                     "ref_boxAggregate", "ref_findCross", "ref_aggregate_cost_horizontal",
                     "ref_cross_stereo_aggregation", "ref_disp_refinement", "ref_calcProxWeight",
                     "ref_computeWeights", "ref_calcAWCostL2R", "ref_calcAWCostR2L", "ref_WTA",
                     "ref_WTA_NCC", "ref_cross_check"]:
            getattr(r, name).restype = None
        r.ref_pixelBasedCostL2R_Color_trunc.argtypes = [_p, _p, _p, _i, _i, _i, _f, _i]
        r.ref_pixelBasedR2L_Color_trunc.argtypes = [_p, _p, _p, _i, _i, _i, _f, _i]
        r.ref_combineCost.argtypes = [_p, _p, _f, _f, _i, _i, _i]
        r.ref_calcProxWeight.argtypes = [_p, _f, _i]
        r.ref_computeWeights.argtypes = [_p, _p, _p, _f, _i, _i, _i]
        _REF = r
    return _REF


def ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the oracle must be C-contiguous"
    return a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------------------
# numpy-level wrappers of the restatement (names follow seq/*.h)

def ad_gray(ref, tar, D, direction=L2R):
    H, W = ref.shape
    out = np.empty((H, W, D), np.float32)
    lib().orc_ad_gray(ptr(ref), ptr(tar), ptr(out), D, H, W, direction)
    return out


def ad_float(ref, tar, D, direction=L2R):
    H, W = ref.shape
    out = np.empty((H, W, D), np.float32)
    lib().orc_ad_float(ptr(ref), ptr(tar), ptr(out), D, H, W, direction)
    return out


def ad_color(ref, tar, D, direction=L2R, trunc=None, norm=0):
    H, W, _ = ref.shape
    out = np.empty((H, W, D), np.float32)
    lib().orc_ad_color(ptr(ref), ptr(tar), ptr(out), D, H, W, direction,
                       0 if trunc is None else 1, 0.0 if trunc is None else float(trunc), norm)
    return out


def census(img, hrad=4, wrad=3):
    H, W = img.shape
    out = np.empty((H, W, (2 * hrad + 1) * (2 * wrad + 1)), np.uint8)
    lib().orc_census(ptr(img), ptr(out), hrad, wrad, H, W)
    return out


def hamming(bref, btar, D, hrad=4, wrad=3):
    H, W, _ = bref.shape
    out = np.empty((H, W, D), np.float32)
    lib().orc_hamming(ptr(bref), ptr(btar), ptr(out), hrad, wrad, H, W, D)
    return out


def rank(img, rad):
    H, W = img.shape
    out = np.empty((H, W), np.uint8)
    lib().orc_rank(ptr(img), ptr(out), rad, H, W)
    return out


def convolve(img, mask, hrad, wrad):
    H, W = img.shape
    out = np.empty((H, W), np.float32)
    m = np.ascontiguousarray(mask, np.float32)
    lib().orc_convolve(ptr(img), ptr(out), ptr(m), H, W, hrad, wrad)
    return out


def ncc(ref, tar, D, hrad, wrad, fill=0.0):
    H, W = ref.shape
    out = np.full((H, W, D), fill, np.float32)
    lib().orc_ncc(ptr(ref), ptr(tar), ptr(out), D, H, W, hrad, wrad)
    return out


def combine(c1, c2, lambda1, lambda2):
    H, W, D = c1.shape
    out = np.array(c1, np.float32, copy=True)
    lib().orc_combine(ptr(out), ptr(np.ascontiguousarray(c2)), lambda1, lambda2, H, W, D)
    return out


def box(cost, rad, inplace=False):
    H, W, D = cost.shape
    if inplace:
        out = np.array(cost, np.float32, copy=True)
        lib().orc_box_inplace(ptr(out), H, W, D, rad)
        return out
    out = np.empty_like(cost)
    lib().orc_box(ptr(np.ascontiguousarray(cost)), ptr(out), H, W, D, rad)
    return out


def median(img, k=3):
    """Median filter of a [H][W] or [H][W][3] u8 image (k odd, borders replicated)."""
    img = np.ascontiguousarray(img, np.uint8)
    H, W = img.shape[:2]
    ch = 1 if img.ndim == 2 else img.shape[2]
    out = np.empty_like(img)
    lib().orc_median(ptr(img), ptr(out), H, W, ch, k)
    return out


def find_cross(rgb, L=17, tau=20):
    H, W, _ = rgb.shape
    horz = np.empty((H, W, 2), np.int32)
    vert = np.empty((H, W, 2), np.int32)
    lib().orc_find_cross(ptr(rgb), ptr(horz), ptr(vert), H, W, L, tau)
    return horz, vert


def prefix_h(cost):
    H, W, D = cost.shape
    out = np.array(cost, np.float32, copy=True)
    lib().orc_prefix_h(ptr(out), H, W, D)
    return out


def cross_aggr(pre, hr, ht, vr, vt):
    H, W, D = pre.shape
    out = np.empty_like(pre)
    lib().orc_cross_aggr(ptr(pre), ptr(out), ptr(hr), ptr(ht), ptr(vr), ptr(vt), H, W, D)
    return out


def prox_weight(gamma_p, rad):
    out = np.empty(((2 * rad + 1) ** 2,), np.float32)
    lib().orc_prox_weight(ptr(out), gamma_p, rad)
    return out


def compute_weights(pw, lab, gamma_s, rad):
    H, W, _ = lab.shape
    out = np.empty((H, W, (2 * rad + 1) ** 2), np.float32)
    lib().orc_compute_weights(ptr(out), ptr(pw), ptr(lab), gamma_s, H, W, rad)
    return out


def aw_l2r(wref, wtar, cost, rad):
    H, W, D = cost.shape
    out = np.empty_like(cost)
    lib().orc_aw_l2r(ptr(wref), ptr(wtar), ptr(cost), ptr(out), H, W, D, rad)
    return out


def aw_l2r_rows(lab_ref, lab_tar, cost, rows, rad, gamma_s, gamma_p):
    """Rows `rows` of the left-to-right adaptive-weight aggregation of the whole
    volume `cost`, with only those rows' weights made (a 1920x1080 image's full
    weight arrays would take 9 GB each).  Returns [len(rows)][W][D]."""
    H, W, D = cost.shape
    cost = np.ascontiguousarray(cost, np.float32)
    pw = prox_weight(gamma_p, rad)
    area = pw.size
    out = np.empty((len(rows), W, D), np.float32)
    for i, y in enumerate(rows):
        wr = np.empty((W, area), np.float32)
        wt = np.empty((W, area), np.float32)
        lib().orc_compute_weights_rows(ptr(wr), ptr(pw), ptr(lab_ref), gamma_s, H, W, rad, int(y), 1)
        lib().orc_compute_weights_rows(ptr(wt), ptr(pw), ptr(lab_tar), gamma_s, H, W, rad, int(y), 1)
        lib().orc_aw_l2r_rows(ptr(wr), ptr(wt), ptr(cost), ptr(out[i]), H, W, D, rad, int(y), 1)
    return out


def aw_r2l(wref, wtar, cost, rad, inplace=False):
    H, W, D = cost.shape
    if inplace:
        out = np.array(cost, np.float32, copy=True)
        lib().orc_aw_r2l(ptr(wref), ptr(wtar), ptr(out), H, W, D, rad)
        return out
    out = np.empty_like(cost)
    lib().orc_aw_r2l_oop(ptr(wref), ptr(wtar), ptr(np.ascontiguousarray(cost)), ptr(out), H, W, D, rad)
    return out


def wta(cost, argmax=False):
    H, W, D = cost.shape
    out = np.empty((H, W), np.uint8)
    lib().orc_wta(ptr(np.ascontiguousarray(cost)), ptr(out), H, W, D, 1 if argmax else 0)
    return out


def cross_check(dref, dtar):
    H, W = dref.shape
    out = np.empty((H, W), np.uint8)
    lib().orc_cross_check(ptr(dref), ptr(dtar), ptr(out), H, W)
    return out


def disp_refinement(disp, horz, vert, D, inplace=False):
    H, W = disp.shape
    if inplace:
        out = np.array(disp, np.uint8, copy=True)
        lib().orc_disp_refinement(ptr(out), ptr(horz), ptr(vert), H, W, D)
        return out
    out = np.empty_like(disp)
    lib().orc_disp_refinement_oop(ptr(np.ascontiguousarray(disp)), ptr(out), ptr(horz), ptr(vert), H, W, D)
    return out


def f64_combine(c1, c2, lambda1, lambda2):
    out = np.empty(c1.shape, np.float64)
    lib().orc64_combine(ptr(c1), ptr(c2), float(lambda1), float(lambda2), c1.size, ptr(out))
    return out


def f64_aw_l2r(labr, labt, cost, rad, gamma_s, gamma_p):
    H, W, D = cost.shape
    out = np.empty(cost.shape, np.float64)
    lib().orc64_aw_l2r(ptr(labr), ptr(labt), ptr(cost), ptr(out), H, W, D, rad, gamma_s, gamma_p)
    return out


def f64_aw_l2r_pre(labr, labt, cost64, rad, gamma_s, gamma_p):
    """FP64 adaptive-weight aggregation of an FP64 volume (weights made once per pixel)."""
    cost64 = np.ascontiguousarray(cost64, np.float64)
    H, W, D = cost64.shape
    out = np.empty_like(cost64)
    if lib().orc64_aw_l2r_pre(ptr(labr), ptr(labt), ptr(cost64), ptr(out), H, W, D, rad, gamma_s, gamma_p) != 0:
        raise MemoryError("orc64_aw_l2r_pre")
    return out


def f64_ncc(ref, tar, D, hrad, wrad):
    H, W = ref.shape
    out = np.empty((H, W, D), np.float64)
    lib().orc64_ncc(ptr(ref), ptr(tar), ptr(out), D, H, W, hrad, wrad)
    return out


def f64_convolve(img, mask, hrad, wrad):
    H, W = img.shape
    out = np.empty((H, W), np.float64)
    m = np.ascontiguousarray(mask, np.float32)
    lib().orc64_convolve(ptr(img), ptr(out), ptr(m), H, W, hrad, wrad)
    return out


LOG5x5 = np.array([0.0239, 0.046, 0.0499, 0.046, 0.0239,
                   0.046, 0.0061, -0.0923, 0.0061, 0.046,
                   0.0499, -0.0923, -0.3182, -0.0923, 0.0499,
                   0.046, 0.0061, -0.0923, 0.0061, 0.046,
                   0.0239, 0.046, 0.0499, 0.046, 0.0239], np.float32)


def params(**kw) -> OrcParams:
    """Pipeline parameters with the reference driver's defaults
    (seq/Main.cpp:102-128): census 9x7, rank radius 7, NCC radius 1, box
    radius 1, adaptive weight radius 16 / gamma_s 7 / gamma_p 36, cross arm
    17 / tau 20 (seq/CrossBasedAggregation.h:8-9), AD truncation 24."""
    p = OrcParams(cost1=1, cost2=3, aggr=3, lambda1=10.0, lambda2=10.0, D=16,
                  census_hrad=4, census_wrad=3, rank_rad=7, ncc_hrad=1, ncc_wrad=1,
                  box_rad=1, aw_rad=16, aw_gamma_s=7.0, aw_gamma_p=36.0,
                  cross_L=17, cross_tau=20, ad_trunc=24.0, right_view=1, box_inplace=0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def pipeline(p: OrcParams, lgray, rgray, lrgb, rrgb, llab=None, rlab=None, want_cost=False):
    """Whole-pair pipeline; returns (disp_left, disp_right, mask, cost_left)."""
    H, W = lgray.shape
    dl = np.zeros((H, W), np.uint8)
    dr = np.zeros((H, W), np.uint8)
    mk = np.zeros((H, W), np.uint8)
    cost = np.empty((H, W, p.D), np.float32) if want_cost else None
    rc = lib().orc_pipeline(C.byref(p), H, W, ptr(lgray), ptr(rgray), ptr(lrgb), ptr(rrgb),
                            ptr(llab) if llab is not None else None,
                            ptr(rlab) if rlab is not None else None,
                            ptr(dl), ptr(dr), ptr(mk), ptr(cost) if cost is not None else None)
    if rc != 0:
        raise RuntimeError("oracle pipeline failed (bad parameters or out of memory)")
    return dl, dr, mk, cost


def view_cost(p: OrcParams, lgray, rgray, lrgb, rrgb):
    """The left view's matching cost volume (cost1, cost2 combined), [H][W][D]."""
    H, W = lgray.shape
    out = np.empty((H, W, p.D), np.float32)
    if lib().orc_view_cost(C.byref(p), H, W, ptr(lgray), ptr(rgray), ptr(lrgb), ptr(rrgb), ptr(out)) != 0:
        raise RuntimeError("oracle view cost failed")
    return out


def set_threads(n: int) -> None:
    """Host threads for the oracle's row loops (n <= 0: all processors)."""
    lib().orc_set_threads(int(n))


def threads() -> int:
    return int(lib().orc_threads())


def synth_pair(seed: int, width: int, height: int, max_disp: int, n_rects: int, n_planes: int = 0,
               sigma: float = 2.0, bg_disp: int = 4):
    """Seeded random-dot pair (left_gray, right_gray, gt_disp): the library's
    generator restated, for CPU runs that must not load the library."""
    L = np.empty((height, width), np.uint8)
    R = np.empty((height, width), np.uint8)
    G = np.empty((height, width), np.uint8)
    if lib().orc_synth_pair(seed, width, height, max_disp, n_rects, n_planes, sigma, bg_disp, ptr(L), ptr(R),
                            ptr(G)) != 0:
        raise ValueError("orc_synth_pair: bad arguments")
    return L, R, G


def gray_to_rgb(g):
    g = np.ascontiguousarray(g, np.uint8)
    H, W = g.shape
    out = np.empty((H, W, 3), np.uint8)
    lib().orc_gray_to_rgb(ptr(g), ptr(out), W, H)
    return out


def rgb_to_lab(rgb):
    rgb = np.ascontiguousarray(rgb, np.uint8)
    H, W, _ = rgb.shape
    out = np.empty((H, W, 3), np.uint8)
    lib().orc_rgb_to_lab(ptr(rgb), ptr(out), W, H)
    return out


def ref_pipeline(p: OrcParams, lgray, rgray, lrgb, rrgb, llab=None, rlab=None):
    """The whole pair through the reference's own seq/ functions (oracle/_ref) in
    its driver's order (seq/Main.cpp:180-257): the left view, the right view as the
    left-to-right pipeline on the mirrored pair, then cross_check
    (seq/CrossCheck.cpp:10-23).  The reference's findCross has its own constants
    (arm 17, threshold 20) and its boxAggregate works in place.  Returns
    (disp_left, disp_right, mask).  Used as the timed CPU baseline where the
    reference build exists."""
    R = reflib()
    if R is None:
        raise RuntimeError("the reference's seq/ build (oracle/_ref) is not present")
    D = p.D

    def view(rg, tg, rc, tc, rl, tl):
        H, W = rg.shape

        def cost(which, trunc):
            o = np.zeros((H, W, D), np.float32)
            if which == 1:  # seq/Main.cpp:183-186
                if trunc:
                    R.ref_pixelBasedCostL2R_Color_trunc(ptr(rc), ptr(tc), ptr(o), D, H, W, p.ad_trunc, 0)
                else:
                    R.ref_pixelBasedCostL2R_Color(ptr(rc), ptr(tc), ptr(o), D, H, W, 0)
            elif which == 2:
                a, b = np.zeros((H, W), np.uint8), np.zeros((H, W), np.uint8)
                R.ref_calculateRankFilt(ptr(rg), ptr(a), p.rank_rad, H, W)
                R.ref_calculateRankFilt(ptr(tg), ptr(b), p.rank_rad, H, W)
                R.ref_pixelBasedL2R(ptr(a), ptr(b), ptr(o), D, H, W)
            elif which == 3:
                nb = (2 * p.census_hrad + 1) * (2 * p.census_wrad + 1)
                a, b = np.zeros((H, W, nb), np.uint8), np.zeros((H, W, nb), np.uint8)
                R.ref_calcCensusTrans(ptr(rg), ptr(a), p.census_hrad, p.census_wrad, H, W)
                R.ref_calcCensusTrans(ptr(tg), ptr(b), p.census_hrad, p.census_wrad, H, W)
                R.ref_calcHammingDist(ptr(a), ptr(b), ptr(o), p.census_hrad, p.census_wrad, H, W, D)
            elif which == 4:
                mask = np.ascontiguousarray(LOG5x5, np.float32)
                a, b = np.zeros((H, W), np.float32), np.zeros((H, W), np.float32)
                R.ref_convolveImage(ptr(rg), ptr(a), ptr(mask), H, W, 2, 2)
                R.ref_convolveImage(ptr(tg), ptr(b), ptr(mask), H, W, 2, 2)
                R.ref_pixelBasedCostL2R_Float(ptr(a), ptr(b), ptr(o), D, H, W)
            elif which == 5:  # den == 0 cells stay as allocated (zero)
                R.ref_calcNCCDispL2R(ptr(rg), ptr(tg), ptr(o), D, H, W, p.ncc_hrad, p.ncc_wrad)
            return o

        c1 = cost(p.cost1, p.aggr == 3)
        if p.cost2:
            R.ref_combineCost(ptr(c1), ptr(cost(p.cost2, False)), p.lambda1, p.lambda2, H, W, D)
        fin = c1
        if p.aggr == 1:
            R.ref_boxAggregate(ptr(c1), H, W, D, p.box_rad)
        elif p.aggr == 2:
            r = p.aw_rad
            pw = np.zeros(((2 * r + 1) ** 2,), np.float32)
            R.ref_calcProxWeight(ptr(pw), p.aw_gamma_p, r)
            wr = np.zeros((H, W, pw.size), np.float32)
            wt = np.zeros((H, W, pw.size), np.float32)
            R.ref_computeWeights(ptr(wr), ptr(pw), ptr(rl), p.aw_gamma_s, H, W, r)
            R.ref_computeWeights(ptr(wt), ptr(pw), ptr(tl), p.aw_gamma_s, H, W, r)
            fin = np.zeros_like(c1)
            R.ref_calcAWCostL2R(ptr(wr), ptr(wt), ptr(c1), ptr(fin), H, W, D, r)
        elif p.aggr == 3:
            arms = [np.zeros((H, W, 2), np.int32) for _ in range(4)]
            R.ref_findCross(ptr(rc), ptr(arms[0]), ptr(arms[2]), H, W)
            R.ref_findCross(ptr(tc), ptr(arms[1]), ptr(arms[3]), H, W)
            R.ref_aggregate_cost_horizontal(ptr(c1), H, W, D)
            fin = np.zeros_like(c1)
            R.ref_cross_stereo_aggregation(ptr(c1), ptr(fin), *[ptr(a) for a in arms], H, W, D)
        win = np.zeros((H, W), np.uint8)
        if p.cost1 == 5 and p.cost2 == 0:
            R.ref_WTA_NCC(ptr(fin), ptr(win), H, W, D)
        else:
            R.ref_WTA(ptr(fin), ptr(win), H, W, D)
        return win

    flip = lambda a: None if a is None else np.ascontiguousarray(a[:, ::-1])
    c = lambda a: None if a is None else np.ascontiguousarray(a)
    dl = view(c(lgray), c(rgray), c(lrgb), c(rrgb), c(llab), c(rlab))
    dr = flip(view(flip(rgray), flip(lgray), flip(rrgb), flip(lrgb), flip(rlab), flip(llab)))
    mk = np.zeros_like(dl)
    H, W = dl.shape
    R.ref_cross_check(ptr(dl), ptr(dr), ptr(mk), H, W)
    return dl, dr, mk
