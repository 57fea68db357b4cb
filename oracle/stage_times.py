"""Per-stage CPU timings of the oracle (the C restatement of the reference's
seq/ code) for the baseline table -- TEST INFRASTRUCTURE ONLY (it times the
oracle; nothing here runs the product library).

Usage:  python oracle/stage_times.py [--out FILE.json]

For each benchmark configuration it times, on one host thread, every stage of
the reference driver's left-view pipeline (seq/Main.cpp:180-257): the matching
costs, CombineCost, the aggregation, WTA, and the cross check of both views.
Large configurations are timed on a strip or crop of the pair and scaled per
cost entry (each printed with its sample).  Two builds are timed: the oracle as
the tests use it (gcc -O2) and the same source with -O3 and the host's own CPU
tuning (-march=native on x86-64, -mcpu=native on aarch64); -ffp-contract=off in
both, so the results are the same.  Then an all-cores figure: one oracle
process per core, each running whole pairs of the mixed 64-pair workload
(pairs i = 0, 1, ... of seeds 0xC3000 + i), as pairs/s.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import multiprocessing as mp
import os
import platform
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402

MIX_SIZES = [(320, 240), (640, 480), (1024, 768), (1280, 720), (1920, 1080)]
MIX_DISP = [32, 64, 128]


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.processor() or platform.machine()


def build_variant(flags, path):
    src = os.path.join(HERE, "rts_oracle.c")
    subprocess.run(["gcc", *flags, "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-o", path, src, "-lm"],
                   check=True, capture_output=True)
    lib = C.CDLL(path)
    for name, args in oracle._ORACLE_SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int if name in oracle._INT_RESULT else None
    return lib


def timed(fn, reps=3):
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts))


def stages(lib, cfg, reps):
    """Seconds per stage on the configuration's sample (one thread)."""
    p = oracle.ptr
    name, W, H, D, c1, c2, ag, extra, (ys, xs) = cfg
    L, Rr, _ = oracle.synth_pair(extra["seed"], W, H, D, extra["rects"], extra["planes"], extra["sigma"], min(4, D - 1))
    L, Rr = np.ascontiguousarray(L[ys, xs]), np.ascontiguousarray(Rr[ys, xs])
    h, w = L.shape
    Lc, Rc = oracle.gray_to_rgb(L), oracle.gray_to_rgb(Rr)
    vol = lambda: np.empty((h, w, D), np.float32)
    out = {}
    c_ad, c_cen, c_comb = vol(), vol(), vol()
    trunc = 1 if ag == 3 else 0
    out["AD colour"] = timed(lambda: lib.orc_ad_color(p(Lc), p(Rc), p(c_ad), D, h, w, 1, trunc, 24.0, 0), reps)
    nb = 63
    bl, br = np.empty((h, w, nb), np.uint8), np.empty((h, w, nb), np.uint8)
    out["census x2"] = timed(lambda: (lib.orc_census(p(L), p(bl), 4, 3, h, w), lib.orc_census(p(Rr), p(br), 4, 3, h, w)),
                             reps)
    out["Hamming"] = timed(lambda: lib.orc_hamming(p(bl), p(br), p(c_cen), 4, 3, h, w, D), reps)

    def combine():
        np.copyto(c_comb, c_ad)
        lib.orc_combine(p(c_comb), p(c_cen), 10.0, 10.0, h, w, D)
    out["CombineCost"] = timed(combine, reps)
    fin = vol()
    if ag == 1:
        out["box 9x9"] = timed(lambda: lib.orc_box(p(c_comb), p(fin), h, w, D, 4), reps)
    elif ag == 2:
        r = 16
        pw = oracle.prox_weight(36.0, r)
        lab_l, lab_r = oracle.rgb_to_lab(Lc), oracle.rgb_to_lab(Rc)
        wl = np.empty((h, w, pw.size), np.float32)
        wr = np.empty_like(wl)
        out["computeWeights x2"] = timed(
            lambda: (lib.orc_compute_weights(p(wl), p(pw), p(lab_l), 7.0, h, w, r),
                     lib.orc_compute_weights(p(wr), p(pw), p(lab_r), 7.0, h, w, r)), 1)
        out["calcAWCostL2R"] = timed(lambda: lib.orc_aw_l2r(p(wl), p(wr), p(c_comb), p(fin), h, w, D, r), 1)
    else:
        hl, vl = np.empty((h, w, 2), np.int32), np.empty((h, w, 2), np.int32)
        hr_, vr_ = np.empty_like(hl), np.empty_like(vl)
        out["findCross x2"] = timed(lambda: (lib.orc_find_cross(p(Lc), p(hl), p(vl), h, w, 17, 20),
                                             lib.orc_find_cross(p(Rc), p(hr_), p(vr_), h, w, 17, 20)), reps)
        pre = vol()

        def prefix():
            np.copyto(pre, c_comb)
            lib.orc_prefix_h(p(pre), h, w, D)
        out["horizontal sums"] = timed(prefix, reps)
        out["cross aggregation"] = timed(lambda: lib.orc_cross_aggr(p(pre), p(fin), p(hl), p(hr_), p(vl), p(vr_), h, w, D),
                                         reps)
    win = np.empty((h, w), np.uint8)
    out["WTA"] = timed(lambda: lib.orc_wta(p(fin), p(win), h, w, D, 0), reps)
    mk = np.empty_like(win)
    out["cross check"] = timed(lambda: lib.orc_cross_check(p(win), p(win), p(mk), h, w), reps)
    entries = h * w * D
    total = sum(out.values())
    return {"sample": f"{w}x{h}, D={D} of {W}x{H}", "entries": entries,
            "stages_s": out, "left_view_s": total,
            # both views (the right view is the same work) and the cross check once
            "pair_s_scaled_to_full": (2 * (total - out["cross check"]) + out["cross check"]) * (W * H * D) / entries,
            "MDE_per_s": W * H * D / 1e6 / ((2 * (total - out["cross check"]) + out["cross check"]) * (W * H * D) / entries)}


CONFIGS = [
    # name, W, H, D, cost1, cost2, aggr, generator, (rows, cols) of the sample
    ("c0 384x288 D16 AD+census cross", 384, 288, 16, 1, 3, 3,
     dict(seed=0xC0, rects=6, planes=0, sigma=2.0), (slice(None), slice(None))),
    ("c1 640x480 D64 AD+census AW 33x33", 640, 480, 64, 1, 3, 2,
     dict(seed=0xC1, rects=12, planes=1, sigma=2.0), (slice(0, 40), slice(None))),
    ("c2 1920x1080 D128 AD+census cross", 1920, 1080, 128, 1, 3, 3,
     dict(seed=0xC2, rects=24, planes=2, sigma=3.0), (slice(0, 64), slice(None))),
    ("c2 1920x1080 D128 AD+census box 9x9", 1920, 1080, 128, 1, 3, 1,
     dict(seed=0xC2, rects=24, planes=2, sigma=3.0), (slice(0, 64), slice(None))),
    ("c2 1920x1080 D128 AD+census AW 33x33", 1920, 1080, 128, 1, 3, 2,
     dict(seed=0xC2, rects=24, planes=2, sigma=3.0), (slice(0, 34), slice(0, 480))),
]


def _pair_worker(i):
    import oracle as O
    O.set_threads(1)
    rng = np.random.default_rng(0xC3000)
    for _ in range(i + 1):
        W, H = MIX_SIZES[rng.integers(len(MIX_SIZES))]
        D = MIX_DISP[rng.integers(len(MIX_DISP))]
    L, Rr, _ = O.synth_pair(0xC3000 + i, W, H, D, 6, 0, 2.0, 4)
    t0 = time.perf_counter()
    O.pipeline(O.params(D=D), L, Rr, O.gray_to_rgb(L), O.gray_to_rgb(Rr))
    return W * H * D, time.perf_counter() - t0


def all_cores(n):
    os.environ["OMP_NUM_THREADS"] = "1"
    ctx = mp.get_context("spawn")
    with ctx.Pool(n) as pool:
        t0 = time.perf_counter()
        res = pool.map(_pair_worker, range(n))
        wall = time.perf_counter() - t0
    mean_s = float(np.mean([t for _, t in res]))
    # steady state of a queue of pairs over n processes: n pairs per mean pair time
    return {"processes": n, "pairs_timed": n, "wall_s": wall, "mean_pair_s": mean_s, "pairs_per_s": n / mean_s,
            "MDE_per_s": n * float(np.mean([e for e, _ in res])) / 1e6 / mean_s,
            "what": "pairs 0..n-1 of the mixed workload, one whole pair (both views + cross check) per process; "
                    "pairs/s = processes / mean pair time"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--no-all-cores", action="store_true")
    args = ap.parse_args()
    oracle.build()
    native = "-mcpu=native" if platform.machine() in ("aarch64", "arm64") else "-march=native"
    res = {"cpu": cpu_model(), "nproc": os.cpu_count(), "machine": platform.machine(), "builds": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for tag, flags in (("gcc -O2", ["-O2"]), (f"gcc -O3 {native}", ["-O3", native])):
            lib = build_variant(flags, os.path.join(tmp, tag.replace(" ", "_") + ".so"))
            lib.orc_set_threads(1)
            res["builds"][tag] = {cfg[0]: stages(lib, cfg, args.reps) for cfg in CONFIGS}
            print(json.dumps({tag: {k: round(v["MDE_per_s"], 3) for k, v in res["builds"][tag].items()}}), flush=True)
    if not args.no_all_cores:
        res["all_cores_mixed_pairs"] = all_cores(os.cpu_count() or 1)
        print(json.dumps(res["all_cores_mixed_pairs"]), flush=True)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
