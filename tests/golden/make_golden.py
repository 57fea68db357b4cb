"""Regenerate tests/golden/seq_golden.npz from the reference's own seq/ code.

The reference's seq/*.cpp (everything but the OpenCV driver) is compiled from
its sources by ``make -C oracle ref`` into ``oracle/_ref/libseqref.so``; this
script feeds it seeded inputs and stores inputs and outputs together, so the
fixtures need nothing but numpy to read.  The whole-pipeline cases chain the
reference's functions in the order of seq/Main.cpp:180-257, and make the right
view by running the same chain on horizontally mirrored images.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

OUT = os.path.join(ROOT, "tests", "golden", "seq_golden.npz")

LOG5x5 = np.array([0.0239, 0.046, 0.0499, 0.046, 0.0239, 0.046, 0.0061, -0.0923, 0.0061, 0.046, 0.0499, -0.0923,
                   -0.3182, -0.0923, 0.0499, 0.046, 0.0061, -0.0923, 0.0061, 0.046, 0.0239, 0.046, 0.0499, 0.046,
                   0.0239], np.float32)


def P(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def smooth(a):
    b = a.astype(np.int32)
    H, W = a.shape
    s = np.zeros_like(b)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            s += b[np.clip(np.arange(H) + dy, 0, H - 1)][:, np.clip(np.arange(W) + dx, 0, W - 1)]
    return ((s + 4) // 9).astype(np.uint8)


def stereo_pair(rng, H, W, D, noise=2.0):
    L = smooth(rng.integers(0, 256, (H, W), dtype=np.uint8))
    d = np.full((H, W), min(4, D - 1), np.int32)
    for _ in range(4):
        x0, y0 = rng.integers(0, W), rng.integers(0, H)
        d[y0:y0 + H // 3 + 1, x0:x0 + W // 3 + 1] = rng.integers(0, D)
    xs = np.clip(np.arange(W)[None, :] + d, 0, W - 1)
    R = np.clip(np.round(L[np.arange(H)[:, None], xs] + rng.normal(0, noise, (H, W))), 0, 255).astype(np.uint8)
    return np.ascontiguousarray(L), np.ascontiguousarray(R)


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    import oracle
    R = oracle.reflib()
    assert R is not None, "reference library not built"
    g = {}
    rng = np.random.default_rng(20240613)

    def vol(H, W, D):
        return np.zeros((H, W, D), np.float32)

    # ---- matching costs on an odd-sized pair ----
    H, W, D = 23, 37, 16
    L, Rg = stereo_pair(rng, H, W, D)
    Lc = np.ascontiguousarray(np.stack([L, smooth(rng.integers(0, 256, (H, W), dtype=np.uint8)), L], -1))
    Rc = np.ascontiguousarray(np.stack([Rg, Rg, smooth(rng.integers(0, 256, (H, W), dtype=np.uint8))], -1))
    g["img/L"], g["img/R"], g["img/Lc"], g["img/Rc"] = L, Rg, Lc, Rc
    for name in ("pixelBasedL2R", "pixelBasedR2L"):
        o = vol(H, W, D); getattr(R, "ref_" + name)(P(L), P(Rg), P(o), D, H, W); g[name] = o
    for norm in (0, 1):
        o = vol(H, W, D); R.ref_pixelBasedCostL2R_Color(P(Lc), P(Rc), P(o), D, H, W, norm); g[f"L2R_Color/n{norm}"] = o
        o = vol(H, W, D); R.ref_pixelBasedR2L_Color(P(Lc), P(Rc), P(o), D, H, W, norm); g[f"R2L_Color/n{norm}"] = o
        o = vol(H, W, D); R.ref_pixelBasedCostL2R_Color_trunc(P(Lc), P(Rc), P(o), D, H, W, 24.0, norm)
        g[f"L2R_Color_trunc24/n{norm}"] = o
        o = vol(H, W, D); R.ref_pixelBasedR2L_Color_trunc(P(Lc), P(Rc), P(o), D, H, W, 24.0, norm)
        g[f"R2L_Color_trunc24/n{norm}"] = o
    Lf = np.zeros((H, W), np.float32); R.ref_convolveImage(P(L), P(Lf), P(LOG5x5), H, W, 2, 2)
    Rf = np.zeros((H, W), np.float32); R.ref_convolveImage(P(Rg), P(Rf), P(LOG5x5), H, W, 2, 2)
    g["convolveImage/L"], g["convolveImage/R"] = Lf, Rf
    for name in ("pixelBasedCostL2R_Float", "pixelBasedCostR2L_Float"):
        o = vol(H, W, D); getattr(R, "ref_" + name)(P(Lf), P(Rf), P(o), D, H, W); g[name] = o
    for hr, wr in ((4, 3), (2, 5)):
        nb = (2 * hr + 1) * (2 * wr + 1)
        bl = np.zeros((H, W, nb), np.uint8); R.ref_calcCensusTrans(P(L), P(bl), hr, wr, H, W)
        br = np.zeros((H, W, nb), np.uint8); R.ref_calcCensusTrans(P(Rg), P(br), hr, wr, H, W)
        o = vol(H, W, D); R.ref_calcHammingDist(P(bl), P(br), P(o), hr, wr, H, W, D)
        g[f"census{hr}x{wr}/L"], g[f"census{hr}x{wr}/R"], g[f"hamming{hr}x{wr}"] = bl, br, o
    for m in (1, 3, 7):
        o = np.zeros((H, W), np.uint8); R.ref_calculateRankFilt(P(L), P(o), m, H, W); g[f"rank{m}"] = o
    for hr, wr in ((1, 1), (3, 3)):
        o = np.full((H, W, D), -7.0, np.float32); R.ref_calcNCCDispL2R(P(L), P(Rg), P(o), D, H, W, hr, wr)
        g[f"ncc{hr}x{wr}"] = o
    flat = np.full((H, W), 9, np.uint8)
    o = np.full((H, W, D), -7.0, np.float32); R.ref_calcNCCDispL2R(P(flat), P(Rg), P(o), D, H, W, 1, 1)
    g["ncc_flat1x1"] = o
    # ---- combine, box, cross, WTA on the AD(trunc)+census pair ----
    c1 = g["L2R_Color_trunc24/n0"].copy()
    c2 = g["hamming4x3"].copy()
    for l1, l2 in ((10.0, 10.0), (7.0, 30.0)):
        a = c1.copy(); R.ref_combineCost(P(a), P(c2.copy()), l1, l2, H, W, D); g[f"combine/{int(l1)}_{int(l2)}"] = a
    cc = g["combine/10_10"]
    for r in (1, 4):
        a = cc.copy(); R.ref_boxAggregate(P(a), H, W, D, r); g[f"box_inplace{r}"] = a
    hl = np.zeros((H, W, 2), np.int32); vl = np.zeros((H, W, 2), np.int32); R.ref_findCross(P(Lc), P(hl), P(vl), H, W)
    ht = np.zeros((H, W, 2), np.int32); vt = np.zeros((H, W, 2), np.int32); R.ref_findCross(P(Rc), P(ht), P(vt), H, W)
    g["findCross/Lh"], g["findCross/Lv"], g["findCross/Rh"], g["findCross/Rv"] = hl, vl, ht, vt
    pre = cc.copy(); R.ref_aggregate_cost_horizontal(P(pre), H, W, D); g["prefix"] = pre
    o = vol(H, W, D); R.ref_cross_stereo_aggregation(P(pre.copy()), P(o), P(hl), P(ht), P(vl), P(vt), H, W, D)
    g["cross"] = o
    w = np.zeros((H, W), np.uint8); R.ref_WTA(P(o), P(w), H, W, D); g["WTA/cross"] = w
    # a volume with many ties and d=0 minima exercises the winner carry
    tie = np.ascontiguousarray(np.floor(cc * 2.0) / 2.0, np.float32)
    w = np.zeros((H, W), np.uint8); R.ref_WTA(P(tie), P(w), H, W, D); g["WTA/ties"] = w
    w = np.zeros((H, W), np.uint8); R.ref_WTA_NCC(P(tie), P(w), H, W, D); g["WTA_NCC/ties"] = w
    g["WTA/ties_in"] = tie
    dref = g["WTA/cross"]
    dtar = np.ascontiguousarray(np.roll(dref, 1, axis=1))
    m = np.zeros((H, W), np.uint8); R.ref_cross_check(P(dref), P(dtar), P(m), H, W); g["cross_check"] = m
    g["cross_check/tar"] = dtar
    # ---- adaptive weights ----
    Hs, Ws, Ds = 20, 24, 8
    La, Ra = stereo_pair(rng, Hs, Ws, Ds)
    laba = np.ascontiguousarray(np.stack([La, rng.integers(100, 156, (Hs, Ws), dtype=np.uint8),
                                          np.full((Hs, Ws), 128, np.uint8)], -1))
    labb = np.ascontiguousarray(np.stack([Ra, rng.integers(100, 156, (Hs, Ws), dtype=np.uint8),
                                          np.full((Hs, Ws), 128, np.uint8)], -1))
    g["aw/labL"], g["aw/labR"] = laba, labb
    ca = rng.random((Hs, Ws, Ds), dtype=np.float32)
    g["aw/cost"] = ca
    for rad in (3, 7):
        pw = np.zeros(((2 * rad + 1) ** 2,), np.float32); R.ref_calcProxWeight(P(pw), 36.0, rad)
        wl = np.zeros((Hs, Ws, pw.size), np.float32); R.ref_computeWeights(P(wl), P(pw), P(laba), 7.0, Hs, Ws, rad)
        wr = np.zeros((Hs, Ws, pw.size), np.float32); R.ref_computeWeights(P(wr), P(pw), P(labb), 7.0, Hs, Ws, rad)
        o = vol(Hs, Ws, Ds); R.ref_calcAWCostL2R(P(wl), P(wr), P(ca), P(o), Hs, Ws, Ds, rad)
        g[f"aw{rad}/prox"], g[f"aw{rad}/l2r"] = pw, o
        if rad == 3:
            g["aw3/wL"] = wl
            a = ca.copy(); R.ref_calcAWCostR2L(P(wl), P(wr), P(a), Hs, Ws, Ds, rad); g["aw3/r2l_inplace"] = a
    # ---- whole pipelines, composed from the reference's functions ----
    for name, (Hp, Wp, Dp, c_1, c_2, ag) in {
        "pipe_ad_census_cross": (24, 40, 16, 1, 3, 3),
        "pipe_ad_census_box": (20, 36, 8, 1, 3, 1),
        "pipe_rank_census_aw": (18, 30, 6, 2, 3, 2),
    }.items():
        Lp, Rp = stereo_pair(rng, Hp, Wp, Dp)
        dl, dr, mk = ref_pipeline(R, Lp, Rp, Dp, c_1, c_2, ag)
        g[f"{name}/L"], g[f"{name}/R"] = Lp, Rp
        g[f"{name}/disp_left"], g[f"{name}/disp_right"], g[f"{name}/mask"] = dl, dr, mk
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT}: {len(g)} arrays, {os.path.getsize(OUT)} bytes")


def ref_view(R, Lg, Rg, Lc, Rc, Llab, Rlab, D, c_1, c_2, ag, lam=(10.0, 10.0)):
    """seq/Main.cpp:180-257 for one view, calling the reference's functions.
    Box aggregation uses the reference's in-place boxAggregate literally."""
    H, W = Lg.shape

    def cost(which, trunc):
        o = np.zeros((H, W, D), np.float32)
        if which == 1:
            if trunc:
                R.ref_pixelBasedCostL2R_Color_trunc(P(Lc), P(Rc), P(o), D, H, W, 24.0, 0)
            else:
                R.ref_pixelBasedCostL2R_Color(P(Lc), P(Rc), P(o), D, H, W, 0)
        elif which == 2:
            a = np.zeros((H, W), np.uint8); b = np.zeros((H, W), np.uint8)
            R.ref_calculateRankFilt(P(Lg), P(a), 7, H, W); R.ref_calculateRankFilt(P(Rg), P(b), 7, H, W)
            R.ref_pixelBasedL2R(P(a), P(b), P(o), D, H, W)
        elif which == 3:
            a = np.zeros((H, W, 63), np.uint8); b = np.zeros((H, W, 63), np.uint8)
            R.ref_calcCensusTrans(P(Lg), P(a), 4, 3, H, W); R.ref_calcCensusTrans(P(Rg), P(b), 4, 3, H, W)
            R.ref_calcHammingDist(P(a), P(b), P(o), 4, 3, H, W, D)
        return o

    c1 = cost(c_1, ag == 3)
    if c_2:
        c2 = cost(c_2, False)
        R.ref_combineCost(P(c1), P(c2), lam[0], lam[1], H, W, D)
    fin = c1
    if ag == 1:
        R.ref_boxAggregate(P(c1), H, W, D, 1)
    elif ag == 2:
        rad = 16 if min(H, W) > 16 else 5
        pw = np.zeros(((2 * rad + 1) ** 2,), np.float32); R.ref_calcProxWeight(P(pw), 36.0, rad)
        wl = np.zeros((H, W, pw.size), np.float32); R.ref_computeWeights(P(wl), P(pw), P(Llab), 7.0, H, W, rad)
        wr = np.zeros((H, W, pw.size), np.float32); R.ref_computeWeights(P(wr), P(pw), P(Rlab), 7.0, H, W, rad)
        fin = np.zeros_like(c1); R.ref_calcAWCostL2R(P(wl), P(wr), P(c1), P(fin), H, W, D, rad)
    elif ag == 3:
        hl = np.zeros((H, W, 2), np.int32); vl = np.zeros((H, W, 2), np.int32); R.ref_findCross(P(Lc), P(hl), P(vl), H, W)
        ht = np.zeros((H, W, 2), np.int32); vt = np.zeros((H, W, 2), np.int32); R.ref_findCross(P(Rc), P(ht), P(vt), H, W)
        R.ref_aggregate_cost_horizontal(P(c1), H, W, D)
        fin = np.zeros_like(c1)
        R.ref_cross_stereo_aggregation(P(c1), P(fin), P(hl), P(ht), P(vl), P(vt), H, W, D)
    win = np.zeros((H, W), np.uint8)
    R.ref_WTA(P(fin), P(win), H, W, D)
    return win


def gray_lab(g):
    # gray image as Lab: a lookup of the project's CIE formula for gray levels
    from rtstereo_gb300 import gray_to_rgb, rgb_to_lab
    return rgb_to_lab(gray_to_rgb(g))


def ref_pipeline(R, Lg, Rg, D, c_1, c_2, ag):
    flip = lambda a: np.ascontiguousarray(a[:, ::-1])
    rgb = lambda a: np.ascontiguousarray(np.repeat(a[:, :, None], 3, axis=2))
    Llab = gray_lab(Lg) if ag == 2 else None
    Rlab = gray_lab(Rg) if ag == 2 else None
    dl = ref_view(R, Lg, Rg, rgb(Lg), rgb(Rg), Llab, Rlab, D, c_1, c_2, ag)
    fr = ref_view(R, flip(Rg), flip(Lg), rgb(flip(Rg)), rgb(flip(Lg)),
                  flip(Rlab) if Rlab is not None else None, flip(Llab) if Llab is not None else None, D, c_1, c_2, ag)
    dr = flip(fr)
    m = np.zeros_like(dl)
    H, W = dl.shape
    R.ref_cross_check(P(dl), P(dr), P(m), H, W)
    return dl, dr, m


if __name__ == "__main__":
    main()
