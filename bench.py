"""Benchmark of the rtstereo per-frame pipeline on one GB300 (or N replicas).

Default workload (the "plain vs FP16" configuration): one 640x480 random-dot
stereo pair, D=64, AD+census(9x7) cost combined by CombineCost, adaptive-weight
aggregation 33x33 (gamma_s 7, gamma_p 36), WTA for the left view and the right
view (mirrored pipeline), and the left/right cross check.  Metric: MDE/s =
W*H*D per pair-step (both views) / time.

  value        device-resident inputs, rts_pipeline_run(DEVICE) per step, CUDA events
               on the launching stream, L2 flushed (256 MB write) before each step
  e2e          the same call with HOST buffers (pinned): H2D of both images (gray, RGB,
               Lab) and D2H of both disparity maps and the mask inside the timed step
  roofline     the dominant kernel (stage timer around its launches, CUDA events)
  cpu_baseline the CPU oracle on a bounded sample of the same workload
  f16          (default line) the FP16 form of the same pair: MDE/s, ratio to the plain
               form, disparity agreement, cost error against FP64 on sampled rows
  c2_cross_1080p (default line) the 1920x1080, D=128 cross-based pipeline, plain and
               FP16 forms, against the stage model's HBM roofline
  c2_box_1080p (default line) the 1920x1080, D=128 box 9x9 pipeline, plain and FP16
               forms (the FP16 form aggregates once for both views)
  serve        (default line) a Poisson stream of mixed pairs through the serving loop
               at --serve-rate pairs/s: per-size p50/p99 and pairs/s
  --impl reference  the CPU implementation (oracle/_ref if built here, else the oracle
               port) on all host cores, same metric and config; its inputs come from the
               oracle's copy of the generator, so it never loads the library

Multi-GPU (torchrun, N>1): independent pairs per rank (weak scaling, no collective on
the data path); the time reported is the max over ranks.
"""
from __future__ import annotations

import argparse
import collections
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (W, H, D, cost1, cost2, aggr, rects, planes, sigma, seed, extra params)
    "aw_640x480_d64": (640, 480, 64, 1, 3, 2, 12, 1, 2.0, 0xC1, {}),
    "cross_384x288_d16": (384, 288, 16, 1, 3, 3, 6, 0, 2.0, 0xC0, {}),
    "cross_1920x1080_d128": (1920, 1080, 128, 1, 3, 3, 24, 2, 3.0, 0xC2, {}),
    "cross_1280x720_d128": (1280, 720, 128, 1, 3, 3, 24, 2, 3.0, 0xC2, {}),
    "census_cross_1280x720_d128": (1280, 720, 128, 3, 0, 3, 24, 2, 3.0, 0xC2, {}),
    "aw_1920x1080_d128": (1920, 1080, 128, 1, 3, 2, 24, 2, 3.0, 0xC2, {}),
    "rank_census_cross_1920x1080_d128": (1920, 1080, 128, 2, 3, 3, 24, 2, 3.0, 0xC2, {"rank_rad": 3}),
    "box_1920x1080_d128": (1920, 1080, 128, 1, 3, 1, 24, 2, 3.0, 0xC2, {"box_rad": 4}),
    "log_census_cross_1920x1080_d128": (1920, 1080, 128, 4, 3, 3, 24, 2, 3.0, 0xC2, {}),
    "census_cross_1920x1080_d128": (1920, 1080, 128, 3, 0, 3, 24, 2, 3.0, 0xC2, {}),
    "ncc_box_1920x1080_d128": (1920, 1080, 128, 5, 0, 1, 24, 2, 3.0, 0xC2, {"box_rad": 4, "ncc_hrad": 3,
                                                                            "ncc_wrad": 3}),
    # smaller cases of the same pipelines (profiling)
    "ncc_box_1280x720_d128": (1280, 720, 128, 5, 0, 1, 24, 2, 3.0, 0xC2, {"box_rad": 4, "ncc_hrad": 3,
                                                                          "ncc_wrad": 3}),
    "log_census_cross_1280x720_d128": (1280, 720, 128, 4, 3, 3, 24, 2, 3.0, 0xC2, {}),
}
DEFAULT = "aw_640x480_d64"


def make_inputs(name, gen=None):
    """The workload's pair and its colour / Lab images.  gen: a module with
    synth_pair / gray_to_rgb / rgb_to_lab -- the library (default), or the
    oracle's restatement of the same generator for the CPU reference arm, which
    must not load the library (the two are bit-identical, tests/test_oracle_synth.py)."""
    if gen is None:
        import rtstereo_gb300 as gen
    W, H, D, c1, c2, ag, rects, planes, sigma, seed, extra = WORKLOADS[name]
    L, Rr, _ = gen.synth_pair(seed, W, H, D, rects, planes, sigma, min(4, D - 1))
    Lc, Rc = gen.gray_to_rgb(L), gen.gray_to_rgb(Rr)
    Ll, Rl = gen.rgb_to_lab(Lc), gen.rgb_to_lab(Rc)
    return (W, H, D, c1, c2, ag, extra), (L, Rr, Lc, Rc, Ll, Rl)


def workload_config(name, precision, world):
    """The `config` object of a bench line; the GPU arm and the CPU reference arm
    print the same one for the same workload."""
    W, H, D, c1, c2, ag = WORKLOADS[name][:6]
    return {"workload": name, "width": W, "height": H, "disp_range": D,
            "pipeline": "cost1=%d cost2=%d aggr=%d, both views + cross check" % (c1, c2, ag),
            "precision": precision, "l2": "flushed (256 MB write) before every timed step",
            "parallelism": f"replicas{world}"}


def f64_aw_rows(L, Rr, Lc, Rc, Ll, Rl, D, rad, gamma_s, gamma_p, lam1, lam2, rows, hr, wr):
    """FP64 adaptive-weight costs of the left view on a few rows, in numpy: the
    same terms as the pipeline (colour SAD and census 9x7 Hamming distance, both
    exact integers, combined as (1 - exp(-a/l1)) + (1 - exp(-h/l2)), then the
    weighted average over the (2 rad + 1)^2 window), every operation in double."""
    H, W = L.shape
    ys, xs = np.arange(H), np.arange(W)

    def census(img):
        # the census code of every pixel packed into a u64 (strict centre > neighbour)
        g = img.astype(np.int16)
        code = np.zeros((H, W), np.uint64)
        k = 0
        for dy in range(-hr, hr + 1):
            for dx in range(-wr, wr + 1):
                code |= (g > g[(ys + dy) % H][:, (xs + dx) % W]).astype(np.uint64) << np.uint64(k)
                k += 1
        return code

    pop8 = np.array([bin(i).count("1") for i in range(256)], np.int32)
    cl, cr = census(L), census(Rr)
    dys, dxs = np.meshgrid(np.arange(-rad, rad + 1), np.arange(-rad, rad + 1), indexing="ij")
    dys, dxs = dys.ravel(), dxs.ravel()
    prox = np.exp(-np.sqrt((dys * dys + dxs * dxs).astype(np.float64)) / gamma_p)
    out = np.empty((len(rows), W, D))
    for i, y in enumerate(rows):
        band = (y + np.arange(-rad, rad + 1)) % H
        # combined costs of the band's rows: [row][x][d]
        xt = (xs[:, None] - np.arange(D)[None, :]) % W
        sad = np.abs(Lc[band][:, :, None, :].astype(np.int32) - Rc[band][:, xt, :].astype(np.int32)).sum(-1)
        ham = pop8[(cl[band][:, :, None] ^ cr[band][:, xt]).view(np.uint8)].reshape(len(band), W, D, 8).sum(-1)
        cost = (1.0 - np.exp(-sad / lam1)) + (1.0 - np.exp(-ham / lam2))

        def weights(lab):
            yy, xx = y + dys[None, :], xs[:, None] + dxs[None, :]
            ok = (yy >= 0) & (yy < H) & (xx >= 0) & (xx < W)
            q = lab[np.clip(yy, 0, H - 1), np.clip(xx, 0, W - 1)].astype(np.float64)
            e = np.sqrt(((q - lab[y][:, None, :].astype(np.float64)) ** 2).sum(-1))
            return np.where(ok, prox[None, :] * np.exp(-e / gamma_s), 0.0)

        wr_, wt_ = weights(Ll), weights(Rl)
        rpos = dys + rad
        cols = (xs[:, None] + dxs[None, :]) % W
        for d in range(D):
            w = wr_ * wt_[(xs - d) % W]
            c = cost[rpos[None, :], cols, d]
            out[i, :, d] = (w * c).sum(1) / w.sum(1)
    return out


def aw_cost_error_vs_f64(ctx, R, p16, p32, L, Rr, Lc, Rc, Ll, Rl):
    """Max error of the FP16 form's (and the plain form's) final left cost volume
    against FP64, relative to the largest FP64 cost, on four sampled rows."""
    H, W = L.shape
    D = p16.disp_range
    rows = [H // 8, 3 * H // 8, 5 * H // 8, 7 * H // 8]
    got = {}
    for k, p in (("f16", p16), ("f32", p32)):
        pr = R.params(**{f: getattr(p, f) for f, _ in R.Params._fields_})
        pr.right_view = 0
        got[k] = ctx.pipeline(pr, L, Rr, Lc, Rc, Ll, Rl, want_cost=True)[3][rows]
    ref = f64_aw_rows(L, Rr, Lc, Rc, Ll, Rl, D, p16.aw_rad, p16.aw_gamma_s, p16.aw_gamma_p, p16.lambda1, p16.lambda2,
                      rows, p16.census_hrad, p16.census_wrad)
    scale = float(np.abs(ref).max())
    return {"rows": rows, "f16_max_abs": float(np.abs(got["f16"] - ref).max()),
            "f16_max_rel": float(np.abs(got["f16"] - ref).max() / scale),
            "f32_max_rel": float(np.abs(got["f32"] - ref).max() / scale)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


# ---------------------------------------------------------------------------
# replicas under torchrun: one process per GPU, each with its own pairs (no data
# exchange); the job's time is the slowest rank's, its work the sum of the ranks'

def dist_init(world):
    import torch
    import torch.distributed as dist
    if world > 1 and not dist.is_initialized():
        # nccl on GPUs; RTS_DIST_BACKEND=gloo runs the same host logic on CPUs
        dist.init_process_group(os.environ.get("RTS_DIST_BACKEND", "nccl"))
    return torch


def _reduce(vals, world, op):
    if world <= 1:
        return [float(v) for v in vals]
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in vals], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return [float(v) for v in t.tolist()]


def ranks_max(vals, world):
    import torch.distributed as dist
    return _reduce(vals, world, dist.ReduceOp.MAX if world > 1 else None)


def ranks_sum(vals, world):
    import torch.distributed as dist
    return _reduce(vals, world, dist.ReduceOp.SUM if world > 1 else None)


def ranks_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def ranks_done(world):
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


class CpuSampler:
    """Times the CPU pipeline on `threads` strips of `rows` rows each of the
    workload's pair, one strip per worker process of a pool made once (its start
    is outside every timed sample).  Workers run the oracle single-threaded."""

    def __init__(self, name, rows, threads, gen=None):
        import multiprocessing as mp
        (W, H, D, c1, c2, ag, extra), imgs = make_inputs(name, gen)
        # a strip keeps every window inside one wrap of its rows (the reference's
        # adaptive-weight loops wrap once, seq/AdaptiveWeightAggregation.cpp:91-93)
        rad = extra.get("aw_rad", 16) if ag == 2 else 0
        rows = min(max(rows, rad + 1), H)
        self.strips = []
        for t in range(threads):
            y0 = (t * rows) % max(1, H - rows + 1)
            self.strips.append(tuple(np.ascontiguousarray(a[y0:y0 + rows]) for a in imgs))
        self.name, self.threads = name, threads
        self.mde = threads * W * rows * D / 1e6
        self.sample = f"{threads} x ({W}x{rows} strip, D={D}, full pipeline both views + cross check)"
        os.environ["OMP_NUM_THREADS"] = "1"  # inherited by the spawned workers
        self.pool = mp.get_context("spawn").Pool(threads)
        self.pool.starmap(_cpu_warm, [() for _ in range(threads)])

    def run(self):
        """One timed sample: (MDE/s, seconds)."""
        t0 = time.perf_counter()
        self.pool.starmap(_cpu_worker, [(self.name, s) for s in self.strips])
        dt = time.perf_counter() - t0
        return self.mde / dt, dt

    def close(self):
        self.pool.close()
        self.pool.join()


def _cpu_warm():
    import oracle
    oracle.lib()


def _cpu_worker(name, strip):
    """One strip through the reference's own seq/ functions in its driver's order
    where that build exists (oracle/_ref), else through the oracle's restatement."""
    import oracle
    W, H, D, c1, c2, ag, rects, planes, sigma, seed, extra = WORKLOADS[name]
    L, Rr, Lc, Rc, Ll, Rl = strip
    p = oracle.params(cost1=c1, cost2=c2, aggr=ag, D=D, box_inplace=1, **extra)
    if oracle.have_reference():
        oracle.ref_pipeline(p, L, Rr, Lc, Rc, Ll, Rl)
    else:
        oracle.pipeline(p, L, Rr, Lc, Rc, Ll, Rl)


def run_reference(args, rank, world):
    name = args.workload
    if rank != 0:
        return
    import oracle
    oracle.build()
    kind = "reference" if oracle.have_reference() else "port"
    threads = os.cpu_count() or 1
    # inputs from the oracle's copy of the generator: this arm never loads the library
    cs = CpuSampler(name, args.cpu_rows, threads, gen=oracle)
    vals = []
    try:
        for i in range(args.warmup + args.steps):
            mde, dt = cs.run()
            if i >= args.warmup:
                vals.append((mde, dt))
    finally:
        cs.close()
    mde = float(np.mean([v[0] for v in vals]))
    ms = float(np.mean([v[1] for v in vals]) * 1000)
    line = {"impl": "reference", "metric": "MDE/s", "value": mde, "unit": "MDE/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic random-dot stereo pair (seeded, no dataset)",
            "config": workload_config(name, args.precision, world),
            "cpu_baseline": {"value": mde, "unit": "MDE/s", "cores": threads, "kind": kind, "sample": cs.sample},
            "e2e": {"value": mde, "unit": "MDE/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if kind == "port":
        line["note"] = "the reference's seq/ sources are not present on this host; the C oracle port is timed"
    print(json.dumps(line), flush=True)


MIX_SIZES = [(320, 240), (640, 480), (1024, 768), (1280, 720), (1920, 1080)]
MIX_DISP = [32, 64, 128]


def mixed_pairs(n, seed0):
    """n random-dot pairs with sizes and disparity ranges drawn from the mixed set."""
    import rtstereo_gb300 as R
    rng = np.random.default_rng(seed0)
    out = []
    for i in range(n):
        W, H = MIX_SIZES[rng.integers(len(MIX_SIZES))]
        D = MIX_DISP[rng.integers(len(MIX_DISP))]
        L, Rr, _ = R.synth_pair(seed0 + i, W, H, D, 6, 0, 2.0, 4)
        out.append((L, Rr, D))
    return out


def run_batch(args, rank, world):
    """64 mixed pairs through rts_batch_run (one launch per stage, CUDA graph)."""
    import ctypes as C

    import torch

    import rtstereo_gb300 as R
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    dist_init(world)
    prec = R.PREC_F16 if args.precision == "f16" else R.PREC_F32
    data = mixed_pairs(args.pairs, 0xC3000 + 1000 * rank)
    ctx = R.Context(dev)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    keep, pairs, params, outs = [], [], [], []
    mde = 0.0
    for L, Rr, D in data:
        H, W = L.shape
        dl, dr = torch.from_numpy(L).cuda(), torch.from_numpy(Rr).cuda()
        o = [torch.empty((H, W), dtype=torch.uint8, device="cuda") for _ in range(3)]
        keep += [dl, dr] + o
        pairs.append(R.Pair(W, H, dl.data_ptr(), dr.data_ptr(), None, None, None, None))
        params.append(R.params(disp_range=D, precision=prec))
        outs.append(R.Out(o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(), None))
        mde += W * H * D / 1e6
    for _ in range(args.warmup):  # the first call autotunes and captures the graph
        ctx.batch_run(pairs, params, outs)
    torch.cuda.synchronize()
    launches0 = ctx.kernel_launches
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    ranks_barrier(world)
    with ClockSampler(dev) as clk:
        for i in range(args.steps):
            flush.zero_()
            evs[i][0].record(stream)
            ctx.batch_run(pairs, params, outs)
            evs[i][1].record(stream)
        torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
    # the plain path for comparison: the same pairs one pipeline run at a time
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    lib = R.lib()
    for _ in range(2):  # warm-up: each shape is tuned and captured on its first run
        for pr, pp, po in zip(pairs, params, outs):
            ctx.check(lib.rts_pipeline_run(ctx.h, R.DEVICE, C.byref(pr), C.byref(pp), C.byref(po)), "pipeline")
    torch.cuda.synchronize()
    t0.record(stream)
    for pr, pp, po in zip(pairs, params, outs):
        ctx.check(lib.rts_pipeline_run(ctx.h, R.DEVICE, C.byref(pr), C.byref(pp), C.byref(po)), "pipeline")
    t1.record(stream)
    torch.cuda.synchronize()
    ms_plain = t0.elapsed_time(t1)
    # whole job: every rank's pairs over the slowest rank's time
    ms, ms_plain = ranks_max([ms, ms_plain], world)
    mde = ranks_sum([mde], world)[0]
    line = {"metric": "MDE/s", "value": mde / (ms / 1e3), "unit": "MDE/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.precision, "data": "synthetic random-dot stereo pairs (seeded)",
            "config": {"workload": "batch_mixed", "pairs": args.pairs, "sizes": MIX_SIZES, "disp": MIX_DISP,
                       "pipeline": "AD+census, cross-based, both views + cross check", "form": "rts_batch_run (graph)"},
            "one_pair_at_a_time_ms": ms_plain, "batch_speedup_vs_one_at_a_time": ms_plain / ms,
            "gpu_launches": ctx.kernel_launches - launches0, "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ranks_done(world)


def latency_target(by_size, size, target_ms):
    """p99 of one size class against a latency target (None if the class is absent)."""
    b = by_size.get(size)
    if not b:
        return None
    return {"size": size, "n": b["n"], "target_ms": target_ms, "p99_ms": b["p99"],
            "from_arrival_p99_ms": b["from_arrival_p99"], "met": b["p99"] < target_ms}


def serve_measure(ctx, rate, requests, budget_gb, max_batch, priority_pixels, precision, world):
    """A Poisson request stream through rts_server_* (continuous batching), then
    the same arrivals one pair at a time through rts_pipeline_run; returns the
    line's fields (latency per size class, pairs/s, clocks)."""
    import torch

    import rtstereo_gb300 as R
    prec = R.PREC_F16 if precision == "f16" else R.PREC_F32
    pool = mixed_pairs(32, 0xC4000)
    rng = np.random.default_rng(0xC4)
    n = requests
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    choice = rng.integers(len(pool), size=n)
    srv = R.Server(ctx, hbm_budget=int(budget_gb * (1 << 30)), max_inflight=64, max_batch=max_batch,
                   precision=prec, priority_pixels=priority_pixels)
    # result buffers: pinned host arrays the device writes directly, reused once a
    # request has been collected
    free_outs = {}

    def take_outs(H, W):
        lst = free_outs.setdefault((H, W), [])
        return lst.pop() if lst else tuple(torch.empty((H, W), dtype=torch.uint8).pin_memory().numpy()
                                           for _ in range(3))

    def submit(L, Rr, D):
        outs = take_outs(*L.shape)
        return srv.submit(R.params(disp_range=D, precision=prec), L, Rr, outs=outs)

    # warm up: the whole pool in flight at once, twice (kernels of every shape, the
    # server's pinned staging and the result buffers grown past what the stream keeps
    # in flight)
    for _ in range(2):
        warm = [submit(L, Rr, D) for L, Rr, D in pool]
        for t, outs in warm:
            srv.wait(t)
            free_outs[outs[0].shape].append(outs)
    ranks_barrier(world)
    mde = 0.0
    delay = np.zeros(n)  # arrival -> accepted by the server (host side)
    lat, queue, run = np.zeros(n), np.zeros(n), np.zeros(n)
    pending = collections.deque()  # (ticket, request index, result buffers), in submission order

    def collect(t, k, outs):
        sub, start, done = srv.wait(t)
        lat[k], queue[k], run[k] = done - sub, start - sub, done - start
        free_outs[outs[0].shape].append(outs)

    dev = torch.cuda.current_device()
    with ClockSampler(dev) as clk:
        t0 = time.perf_counter()
        i = 0
        while i < n:
            now = time.perf_counter() - t0
            while i < n and arrivals[i] <= now:
                L, Rr, D = pool[choice[i]]
                t, outs = submit(L, Rr, D)
                pending.append((t, i, outs))
                delay[i] = (time.perf_counter() - t0 - arrivals[i]) * 1e3
                mde += L.shape[0] * L.shape[1] * D / 1e6
                i += 1
            srv.progress()
            while pending and srv.poll(pending[0][0]) == 1:
                collect(*pending.popleft())
        while pending:
            collect(*pending.popleft())
        wall = time.perf_counter() - t0
    srv.close()
    # the same arrivals served one pair at a time by the plain call (rts_pipeline_run,
    # HOST buffers, synchronous): latency from arrival, queueing included
    seq_lat = np.zeros(n)
    for L, Rr, D in pool:
        ctx.pipeline(R.params(disp_range=D, precision=prec), L, Rr)  # warm
    t1 = time.perf_counter()
    for k in range(n):
        while time.perf_counter() - t1 < arrivals[k]:
            pass
        L, Rr, D = pool[choice[k]]
        ctx.pipeline(R.params(disp_range=D, precision=prec), L, Rr)
        seq_lat[k] = (time.perf_counter() - t1 - arrivals[k]) * 1e3
    seq_wall = time.perf_counter() - t1
    arr_lat = lat + delay  # from the request's arrival (the host's submit delay added)
    # per size class (the 1920x1080 pairs carry the latency target); the parts of
    # a request's latency: waiting for admission, then launch to completion seen
    # by the host; and the host's delay from the request's arrival to its submit
    sizes = np.array([pool[c][0].shape[1] * 10000 + pool[c][0].shape[0] for c in choice[:len(lat)]])
    by_size = {}
    for code in sorted(set(sizes.tolist())):
        m = sizes == code
        sel = lat[m]
        by_size[f"{code // 10000}x{code % 10000}"] = {
            "n": int(sel.size), "p50": float(np.percentile(sel, 50)), "p99": float(np.percentile(sel, 99)),
            "queue_p99": float(np.percentile(queue[m], 99)), "run_p50": float(np.percentile(run[m], 50)),
            "run_p99": float(np.percentile(run[m], 99)), "submit_delay_p99": float(np.percentile(delay[m], 99)),
            "from_arrival_p99": float(np.percentile(arr_lat[m], 99)),
            "one_at_a_time_p50": float(np.percentile(seq_lat[m], 50)),
            "one_at_a_time_p99": float(np.percentile(seq_lat[m], 99))}
    # whole job: every rank serves its own stream; the job's wall time is the slowest's
    wall = ranks_max([wall], world)[0]
    served, mde = ranks_sum([n, mde], world)
    p99_all = ranks_max([float(np.percentile(lat, 99))], world)[0]
    return {"value": served / wall, "unit": "pairs/s", "wall_s": wall, "requests": n, "offered_per_s": rate,
            "config": {"workload": "serve_poisson", "requests": n, "rate_per_s": rate, "hbm_budget_gb": budget_gb,
                       "max_batch": max_batch, "priority_pixels": priority_pixels, "precision": precision,
                       "outputs": "pinned host arrays, reused", "sizes": MIX_SIZES, "disp": MIX_DISP,
                       "pipeline": "AD+census, cross-based, both views + cross check"},
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "max": float(lat.max()), "from_arrival_p99": float(np.percentile(arr_lat, 99)),
                           "by_size": by_size, "p99_max_over_ranks": p99_all},
            # the latency target of the large size class: p99 under 5 ms per 1920x1080 pair,
            # submit to result (from_arrival adds the host's delay before the submit)
            "latency_target": latency_target(by_size, "1920x1080", 5.0),
            "one_at_a_time": {"unit": "pairs/s", "value": n / seq_wall, "p50_ms": float(np.percentile(seq_lat, 50)),
                              "p99_ms": float(np.percentile(seq_lat, 99)),
                              "what": "the same arrivals, rts_pipeline_run per pair (HOST buffers), latency from arrival"},
            "MDE_per_s": mde / wall, "clocks": clk.summary()}


def run_serve(args, rank, world):
    """Poisson request stream through rts_server_* (continuous batching)."""
    import torch

    import rtstereo_gb300 as R
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    dist_init(world)
    ctx = R.Context(dev)
    r = serve_measure(ctx, args.rate, args.requests, args.budget_gb, args.max_batch, args.priority_pixels,
                      args.precision, world)
    line = {"metric": "pairs/s", "value": r["value"], "unit": "pairs/s", "n_gpus": world, "steps": r["requests"],
            "warmup": 64, "ms_per_step": r["wall_s"] * 1e3 / r["requests"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
            "data": "synthetic random-dot stereo pairs (seeded)", "config": r["config"],
            **{k: r[k] for k in ("latency_ms", "latency_target", "one_at_a_time", "MDE_per_s", "clocks")}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ranks_done(world)


class Bench:
    """One GPU's context and launching stream, and the measurement of one
    workload's pipeline step through the public call (rts_pipeline_run)."""

    def __init__(self, dev, world, steps, warmup):
        import torch

        import rtstereo_gb300 as R
        self.dev, self.world, self.steps, self.warmup = dev, world, steps, warmup
        self.ctx = R.Context(dev)
        # a dedicated (non-default) stream: the library launches on it, the events record on it
        self.stream = torch.cuda.Stream(device=dev)
        torch.cuda.set_stream(self.stream)
        self.ctx.set_stream(self.stream.cuda_stream)
        self.flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
        self.sms = torch.cuda.get_device_properties(dev).multi_processor_count

    def measure(self, name, precision):
        import ctypes as C

        import torch

        import rtstereo_gb300 as R
        dev, world, ctx, stream, flush = self.dev, self.world, self.ctx, self.stream, self.flush
        (W, H, D, c1, c2, ag, extra), imgs = make_inputs(name)
        L, Rr, Lc, Rc, Ll, Rl = imgs
        prec = R.PREC_F16 if precision == "f16" else R.PREC_F32
        p = R.params(cost1=c1, cost2=c2, aggr=ag, disp_range=D, precision=prec, **extra)
        # device-resident inputs and outputs; a pipeline gets the images it reads:
        # the cross-based one gray images only (colour = gray in three channels, as the
        # reference driver reads a gray file), adaptive weights also RGB and Lab
        gray_only = ag == 3
        t = lambda a: torch.from_numpy(a).to(f"cuda:{dev}")
        dL, dR, dLc, dRc, dLl, dRl = (t(a) for a in imgs)
        ptr = lambda a: None if gray_only else a.data_ptr()
        o_dl = torch.empty((H, W), dtype=torch.uint8, device=f"cuda:{dev}")
        o_dr = torch.empty_like(o_dl)
        o_mk = torch.empty_like(o_dl)
        pair = R.Pair(W, H, dL.data_ptr(), dR.data_ptr(), ptr(dLc), ptr(dRc), ptr(dLl), ptr(dRl))
        out = R.Out(o_dl.data_ptr(), o_dr.data_ptr(), o_mk.data_ptr(), None)
        lib = R.lib()

        def step():
            ctx.check(lib.rts_pipeline_run(ctx.h, R.DEVICE, C.byref(pair), C.byref(p), C.byref(out)), "pipeline")

        for _ in range(self.warmup):
            step()
        torch.cuda.synchronize()
        # timed region: per-step events, L2 flushed before each step (outside the events)
        launches0 = ctx.kernel_launches
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(self.steps)]
        ranks_barrier(world)
        torch.cuda.synchronize()
        with ClockSampler(dev) as clk:
            t0 = time.perf_counter()
            for i in range(self.steps):
                flush.zero_()
                evs[i][0].record(stream)
                step()
                evs[i][1].record(stream)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        ranks_barrier(world)
        launches = ctx.kernel_launches - launches0
        ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
        # per-kernel times from the library's stage timer (CUDA events around every
        # launch on the launching stream), on extra steps outside the timed region
        ctx.enable_stage_timing(True)
        ctx.reset_stage_times()
        for i in range(self.steps):
            flush.zero_()
            step()
        torch.cuda.synchronize()
        stages = ctx.stage_times()
        ctx.enable_stage_timing(False)
        ms = ranks_max([ms], world)[0]
        mde_pair = W * H * D / 1e6
        # e2e: HOST (pinned) buffers through the same public call
        pin = lambda a: torch.from_numpy(a).pin_memory()
        hL, hR, hLc, hRc, hLl, hRl = (pin(a) for a in imgs)
        ho = [torch.empty((H, W), dtype=torch.uint8).pin_memory() for _ in range(3)]
        hpair = R.Pair(W, H, hL.data_ptr(), hR.data_ptr(), ptr(hLc), ptr(hRc), ptr(hLl), ptr(hRl))
        hout = R.Out(ho[0].data_ptr(), ho[1].data_ptr(), ho[2].data_ptr(), None)

        def hstep():
            ctx.check(lib.rts_pipeline_run(ctx.h, R.HOST, C.byref(hpair), C.byref(p), C.byref(hout)), "pipeline")

        for _ in range(max(1, self.warmup)):
            hstep()
        e_ms = []
        for i in range(self.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            hstep()
            e_ms.append((time.perf_counter() - t1) * 1e3)
        e2e_ms = ranks_max([float(np.mean(e_ms))], world)[0]
        h2d = sum(a.numel() for a in ((hL, hR) if gray_only else (hL, hR, hLc, hRc, hLl, hRl)))
        # the HOST run's result is the device run's
        agree = bool(np.array_equal(ho[0].numpy(), o_dl.cpu().numpy()))
        peaks, src = measured_peaks()
        roof = roofline(stages, name, W, H, D, ag, peaks, src, p, ms, self.sms)
        return {"name": name, "precision": precision, "params": p, "imgs": imgs, "W": W, "H": H, "D": D, "ag": ag,
                "value": world * mde_pair / (ms / 1e3), "ms": ms, "wall_s": wall, "gpu_launches": launches,
                "e2e": {"value": world * mde_pair / (e2e_ms / 1e3), "unit": "MDE/s", "ms_per_step": e2e_ms,
                        "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 3 * W * H,
                        "host_equals_device_result": agree},
                "stages_ms_per_step": {k: v[1] / self.steps for k, v in stages.items()},
                "roofline": roof, "clocks": clk.summary(), "out": [a.numpy().copy() for a in ho]}


def agreement(a, b):
    """Share of equal disparities (both views) and mask cells of two runs."""
    return {"disp_left": float((a[0] == b[0]).mean()), "disp_right": float((a[1] == b[1]).mean()),
            "mask": float((a[2] == b[2]).mean())}


def c2_cross_record(bench, peaks):
    """The 1920x1080, D=128 cross-based pipeline (plain and FP16 forms) against
    the stage model's HBM roofline."""
    name = "cross_1920x1080_d128"
    m = bench.measure(name, "f32")
    m16 = bench.measure(name, "f16")
    roof = m["roofline"]
    bp = roof["pipeline"]["bytes_per_pair"]
    target_ms = bp / (0.6 * peaks["hbm_gbs"] * 1e9) * 1e3  # 60 % of the measured copy bandwidth
    return {"workload": name, "ms_per_pair": m["ms"], "value": m["value"], "unit": "MDE/s",
            "e2e_ms_per_pair": m["e2e"]["ms_per_step"], "pipeline_frac": roof["pipeline"]["frac"],
            "pipeline_bytes_per_pair": bp, "target": {"frac": 0.6, "ms_per_pair": target_ms,
                                                      "met": m["ms"] <= target_ms},
            "stages_ms_per_step": m["stages_ms_per_step"], "dominant_kernel": roof, "clocks": m["clocks"],
            "f16": {"ms_per_pair": m16["ms"], "value": m16["value"], "ratio_to_plain": m16["value"] / m["value"],
                    "agreement": agreement(m["out"], m16["out"]), "pipeline_frac": m16["roofline"]["pipeline"]["frac"],
                    "stages_ms_per_step": m16["stages_ms_per_step"], "clocks": m16["clocks"]}}


def c2_box_record(bench):
    """The 1920x1080, D=128 box 9x9 pipeline, plain and FP16 forms: the FP16 form
    aggregates once and its box + arg-min kernel also forms the right view's
    minima (x - d), the plain form runs the mirrored pipeline for the right view."""
    name = "box_1920x1080_d128"
    m = bench.measure(name, "f32")
    m16 = bench.measure(name, "f16")
    return {"workload": name, "ms_per_pair": m["ms"], "value": m["value"], "unit": "MDE/s",
            "e2e_ms_per_pair": m["e2e"]["ms_per_step"], "stages_ms_per_step": m["stages_ms_per_step"],
            "dominant_kernel": m["roofline"], "clocks": m["clocks"],
            "f16": {"ms_per_pair": m16["ms"], "value": m16["value"], "ratio_to_plain": m16["value"] / m["value"],
                    "agreement": agreement(m["out"], m16["out"]), "stages_ms_per_step": m16["stages_ms_per_step"],
                    "clocks": m16["clocks"]}}


def f16_record(bench, plain):
    """The FP16 form of the same workload as the line's plain run."""
    import rtstereo_gb300 as R
    m = bench.measure(plain["name"], "f16")
    rec = {"value": m["value"], "unit": "MDE/s", "ms_per_step": m["ms"], "ratio_to_plain": m["value"] / plain["value"],
           "e2e": m["e2e"], "agreement": agreement(plain["out"], m["out"]), "roofline": m["roofline"],
           "stages_ms_per_step": m["stages_ms_per_step"], "clocks": m["clocks"]}
    if plain["ag"] == 2:
        rec["cost_error_vs_f64"] = aw_cost_error_vs_f64(bench.ctx, R, m["params"], plain["params"], *plain["imgs"])
    return rec


def run_modules(args, rank, world):
    """The drop-in module path: the reference driver's left-view chain for
    AD + census, cross-based aggregation (seq/Main.cpp:180-257) called module by
    module through the seq-signature entry points with HOST buffers, as a caller
    of include/rts_seq_compat.hpp does (every call copies its inputs to the device
    and its outputs back, and synchronises).  Beside it the fused pipeline on the
    same pair, left view only, with HOST buffers."""
    import torch

    import rtstereo_gb300 as R
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    name = args.workload
    (W, H, D, c1, c2, ag, extra), (L, Rr, Lc, Rc, Ll, Rl) = make_inputs(name)
    if (c1, c2, ag) != (1, 3, 3):
        raise SystemExit("--module-path: an AD + census, cross-based workload")
    ctx = R.Context(dev)

    def chain(t):
        def timed(key, fn):
            t0 = time.perf_counter()
            v = fn()
            t[key] = t.get(key, 0.0) + (time.perf_counter() - t0) * 1e3
            return v
        ad = timed("pixelBasedCostL2R_Color", lambda: ctx.pixelBasedCostL2R_Color(Lc, Rc, D, trunc=24.0))
        bl = timed("calcCensusTrans x2", lambda: ctx.calcCensusTrans(L))
        br = timed("calcCensusTrans x2", lambda: ctx.calcCensusTrans(Rr))
        hm = timed("calcHammingDist", lambda: ctx.calcHammingDist(bl, br, D))
        cc = timed("combineCost", lambda: ctx.combineCost(ad, hm, 10.0, 10.0))
        hl, vl = timed("findCross x2", lambda: ctx.findCross(Lc))
        hr, vr = timed("findCross x2", lambda: ctx.findCross(Rc))
        pre = timed("aggregate_cost_horizontal", lambda: ctx.aggregate_cost_horizontal(cc))
        agg = timed("cross_stereo_aggregation", lambda: ctx.cross_stereo_aggregation(pre, hl, hr, vl, vr))
        return timed("WTA", lambda: ctx.WTA(agg))

    for _ in range(args.warmup):
        chain({})
    t = {}
    t0 = time.perf_counter()
    for _ in range(args.steps):
        d_mod = chain(t)
    ms = (time.perf_counter() - t0) * 1e3 / args.steps
    p = R.params(disp_range=D, right_view=0)
    for _ in range(args.warmup):
        ctx.pipeline(p, L, Rr)
    t1 = time.perf_counter()
    for _ in range(args.steps):
        d_fused = ctx.pipeline(p, L, Rr)[0]
    ms_fused = (time.perf_counter() - t1) * 1e3 / args.steps
    if rank == 0:
        print(json.dumps({
            "metric": "MDE/s", "value": W * H * D / 1e6 / (ms / 1e3), "unit": "MDE/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic random-dot stereo pair (seeded, no dataset)",
            "config": {"workload": name, "width": W, "height": H, "disp_range": D,
                       "pipeline": "left view, AD(trunc 24)+census, cross-based, WTA; module by module, HOST buffers",
                       "path": "seq-signature module entry points (rts_seq_compat.hpp), host wall clock"},
            "modules_ms_per_step": {k: v / args.steps for k, v in t.items()},
            "fused_left_view_ms": ms_fused, "fused_speedup": ms / ms_fused,
            "same_disparities": bool(np.array_equal(d_mod, d_fused))}), flush=True)


def run_ours(args, rank, world):
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    dist_init(world)
    bench = Bench(dev, world, args.steps, args.warmup)
    m = bench.measure(args.workload, args.precision)
    extra = {}
    # the other target figures ride on the default line (one GPU): the FP16 form,
    # the 1920x1080 cross-based and box pipelines, and the serving loop
    if world == 1 and args.workload == DEFAULT and args.precision == "f32" and not args.no_extra:
        peaks, _ = measured_peaks()
        extra["f16"] = f16_record(bench, m)
        extra["c2_cross_1080p"] = c2_cross_record(bench, peaks)
        extra["c2_box_1080p"] = c2_box_record(bench)
        srv = serve_measure(bench.ctx, args.serve_rate, args.requests, args.budget_gb, args.max_batch,
                            args.priority_pixels, "f16", world)
        extra["serve"] = {k: srv[k] for k in ("value", "unit", "offered_per_s", "requests", "latency_target",
                                              "latency_ms", "one_at_a_time", "config", "clocks")}
    if rank != 0:
        ranks_done(world)
        return
    line = {"metric": "MDE/s", "value": m["value"], "unit": "MDE/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": m["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f16" if args.precision == "f16" else "f32",
            "data": "synthetic random-dot stereo pair (seeded, no dataset)",
            "config": workload_config(args.workload, args.precision, world),
            "e2e": m["e2e"], "gpu_launches": m["gpu_launches"], "wall_s": m["wall_s"],
            "stages_ms_per_step": m["stages_ms_per_step"], "roofline": m["roofline"], "clocks": m["clocks"], **extra}
    if not args.no_cpu:
        import oracle
        cs = CpuSampler(args.workload, args.cpu_rows, 1)
        try:
            mde, dt = cs.run()
        finally:
            cs.close()
        line["cpu_baseline"] = {"value": mde, "unit": "MDE/s", "cores": 1,
                                "kind": "reference" if oracle.have_reference() else "port", "sample": cs.sample,
                                "seconds": dt}
    print(json.dumps(line), flush=True)
    ranks_done(world)


# DRAM bytes per cost entry of the two cross-based kernels, from one ncu capture
# of each at 1280x720, D=128 (one launch covers both views), by form:
# 0 plain (f32 segments), 1 FP16 (f16 segments), 2 integer costs (u16 segments);
# a launch at another size moves these per entry
NCU_BYTES_PER_ENTRY = {("cross_vert_wta", 0): 4.16, ("cross_hseg", 0): 4.00,
                       ("cross_vert_wta", 1): 2.13, ("cross_hseg", 1): 2.00,
                       ("cross_vert_wta", 2): 2.13, ("cross_hseg", 2): 2.00}
# ncu DRAM bytes of one plain-form adaptive-weight launch (k_aw_wta_pipe, one view)
# at 640x480, D=64 (the full capture of that launch)
NCU_AW_BYTES = {(640, 480, 64): 85.31e6}
# the unit that binds k_aw_wta_pipe (plain form) by the same ncu capture: the SM's
# L1/shared-memory data pipe (l1tex__data_pipe_lsu_wavefronts, share of its peak)
NCU_AW_L1_BUSY = {(640, 480, 64): 0.849}
# DRAM bytes (read + write) of one k_box_best_dp launch, ncu at 1920x1080, D=128, r=4
NCU_BOX_BYTES = {(1920, 1080, 128, 4): 1.1375e9}


def roofline(stages, name, W, H, D, ag, peaks, src, p, ms_pair=None, sms=152):
    """Dominant kernel: algorithmic work per launch / its CUDA-event time, against
    the measured peak; traffic = DRAM bytes per launch from ncu."""
    # left_view / right_view are scopes around a view's stages, not kernels
    stages = {k: v for k, v in stages.items() if k not in ("left_view", "right_view")}
    if not stages:
        return None
    dom = max(stages.items(), key=lambda kv: kv[1][1])
    kname, (launches, total_ms) = dom
    per_launch_ms = total_ms / max(1, launches)
    E = W * H * D  # entries per view
    if kname == "aw_wta":
        # one launch = one view.  Per tap per entry the plain form issues 4 FP32-pipe
        # operations (w = wR*wT, sum w, C*w, sum: the reference's order, unfused), the
        # FP16 form 3 (the last two as one fused multiply-add)
        taps = (2 * p.aw_rad + 1) ** 2
        ops_per_tap = 3 if p.precision else 4
        ops = float(ops_per_tap * taps * E)
        achieved = ops / (per_launch_ms / 1e3) / 1e12
        mhz = peaks.get("sm_max_mhz", 2070.0)
        peak = sms * 128 * mhz * 1e6 / 1e12  # one FP32 operation per lane per clock
        traffic = NCU_AW_BYTES.get((W, H, D)) if not p.precision else None
        kern = "k_aw_wta_pipe" if (not p.precision or D % 8 == 0) else "k_aw_wta"
        out = {"bound": "fp32", "kernel": kern, "achieved": achieved, "peak": peak, "unit": "T FP32-pipe op/s",
               "frac": achieved / peak, "traffic": traffic, "launches": launches, "ms_per_launch": per_launch_ms,
               "ops_per_launch": ops, "ops_per_tap": ops_per_tap,
               "peak_source": f"FP32 pipe: {sms} SMs (device attribute) x 128 lanes x {mhz:.0f} MHz "
                              f"({src} max clock), one operation per lane per clock; no tensor-core or HBM "
                              f"bound applies (DRAM < 1% busy)"}
        if not p.precision and (W, H, D) in NCU_AW_L1_BUSY:
            out["binding_unit"] = {"unit": "L1/shared-memory data pipe", "busy_ncu": NCU_AW_L1_BUSY[(W, H, D)],
                                   "note": "16-byte shared loads of weights and costs, colour-distance table reads"}
        return out
    if kname == "box_wta":
        # one launch = one view: (2r+1)^2 sequential FP32 adds per entry (the
        # reference's single chain), no other bound near (the volume read once)
        ops = float((2 * p.box_rad + 1) ** 2 * E)
        achieved = ops / (per_launch_ms / 1e3) / 1e12
        mhz = peaks.get("sm_max_mhz", 2070.0)
        peak = sms * 128 * mhz * 1e6 / 1e12
        return {"bound": "fp32", "kernel": "k_box_best_dp" if (D % 2 == 0 and D > 32) else "k_box_best",
                "achieved": achieved, "peak": peak, "unit": "T FP32-pipe op/s", "frac": achieved / peak,
                "traffic": NCU_BOX_BYTES.get((W, H, D, p.box_rad)), "launches": launches,
                "ms_per_launch": per_launch_ms, "ops_per_launch": ops,
                "peak_source": f"FP32 pipe: {sms} SMs (device attribute) x 128 lanes x {mhz:.0f} MHz "
                               f"({src} max clock), one operation per lane per clock"}
    if kname == "cost" and p.cost1 == 5 and p.cost2 == 0:
        # NCC volume, one stage per view (k_ncc_tiled after the window means): per
        # tap per entry rv*tv, (rv*rv)*tv, ((rv*rv)*tv)*tv and the two sums -- rv,
        # rv*rv and tv are per pixel and tap, shared by every disparity
        taps = (2 * p.ncc_hrad + 1) * (2 * p.ncc_wrad + 1)
        ops = float(5 * taps * E)
        achieved = ops / (per_launch_ms / 1e3) / 1e12
        mhz = peaks.get("sm_max_mhz", 2070.0)
        peak = sms * 128 * mhz * 1e6 / 1e12
        return {"bound": "fp32", "kernel": "k_ncc_tiled", "achieved": achieved, "peak": peak,
                "unit": "T FP32-pipe op/s", "frac": achieved / peak, "traffic": None, "launches": launches,
                "ms_per_launch": per_launch_ms, "ops_per_launch": ops, "ops_per_tap": 5,
                "peak_source": f"FP32 pipe: {sms} SMs (device attribute) x 128 lanes x {mhz:.0f} MHz "
                               f"({src} max clock), one operation per lane per clock; the stage also holds "
                               f"the window means (2-3 % of it)"}
    # HBM stage model (one launch = both views): the cost volume crosses HBM four
    # times per view at S bytes an entry; the row-segment kernel owns the first two
    # crossings (written by matching and combining, read by aggregation), the
    # vertical kernel the last two (written by aggregation, read by WTA)
    # integer costs (census or truncated AD alone) keep u16 segments in both forms
    int_costs = ag == 3 and p.cost2 == 0 and (p.cost1 == 3 or (p.cost1 == 1 and float(p.ad_trunc).is_integer()))
    S = 2 if (p.precision or int_costs) else 4
    views = 2
    byts = views * 2 * S * E
    achieved = byts / (per_launch_ms / 1e3) / 1e9
    peak = peaks["hbm_gbs"]
    bpe = NCU_BYTES_PER_ENTRY.get((kname, 2 if int_costs else 1 if p.precision else 0))
    out = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak, "traffic": bpe * views * E if bpe else None, "launches": launches,
           "ms_per_launch": per_launch_ms, "bytes_per_launch": byts, "peak_source": src}
    if ms_pair:
        # the whole pair against the same model: 2 (4 S E) + 2 (2 W H + 6 W H) + 3 W H bytes
        bp = 2 * (4 * S * E) + 2 * (8 * W * H) + 3 * W * H
        out["pipeline"] = {"bytes_per_pair": bp, "achieved": bp / (ms_pair / 1e3) / 1e9,
                           "frac": bp / (ms_pair / 1e3) / 1e9 / peak}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT, choices=sorted(WORKLOADS) + ["batch_mixed", "serve_poisson"])
    ap.add_argument("--pairs", type=int, default=64, help="batch_mixed: pairs per batch")
    ap.add_argument("--requests", type=int, default=2000, help="serve_poisson: requests in the stream")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve_poisson: Poisson arrival rate (pairs/s)")
    ap.add_argument("--budget-gb", type=float, default=40.0, help="serve_poisson: HBM admitted at once")
    ap.add_argument("--max-batch", type=int, default=2, help="serve_poisson: pairs launched together")
    ap.add_argument("--priority-pixels", type=int, default=1920 * 1080,
                    help="serve_poisson: pairs of at least this many pixels run alone on high-priority streams "
                         "(0: one class)")
    ap.add_argument("--precision", default="f32", choices=["f32", "f16"])
    ap.add_argument("--cpu-rows", type=int, default=None,
                    help="rows per CPU strip (default 48 for the 1-thread baseline, 24 for --impl reference)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--module-path", action="store_true",
                    help="time the drop-in module path (seq-signature calls, HOST buffers) on the workload")
    ap.add_argument("--no-extra", action="store_true",
                    help="default workload: skip the f16 / c2_cross_1080p / c2_box_1080p / serve sub-records")
    ap.add_argument("--serve-rate", type=float, default=600.0,
                    help="offered rate (pairs/s) of the serve sub-record of the default line")
    args = ap.parse_args()
    if args.cpu_rows is None:
        args.cpu_rows = 24 if args.impl == "reference" else 48
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "batch_mixed":
        run_batch(args, rank, world)
    elif args.workload == "serve_poisson":
        run_serve(args, rank, world)
    elif args.module_path:
        run_modules(args, rank, world)
    else:
        run_ours(args, rank, world)


if __name__ == "__main__":
    main()
