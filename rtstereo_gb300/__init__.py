"""rtstereo_gb300 -- GB300 (sm_103a) implementation of rtstereo's per-frame
stereo-matching pipeline behind a C ABI (include/rtstereo.h).

This Python layer is plumbing over the C ABI (ctypes), used by the tests and
the benchmark.  ``Context`` mirrors the reference's seq/ module functions by
name; each method takes numpy arrays in the reference's layouts (HOST memory:
the library copies to the device, runs, copies back) and returns the outputs.
Device-resident use goes through ``Context.call`` with raw device pointers and
``mem=DEVICE``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from ._native import (AGGR_AW, AGGR_BOX, AGGR_CROSS, AGGR_NONE, COST_AD, COST_CENSUS, COST_LOG, COST_NCC,
                      COST_NONE, COST_RANK, DEVICE, HOST, PREC_F16, PREC_F32, Out, Pair, Params, RequestStats,
                      RtsError, ServerConfig)

__all__ = ["Context", "Server", "Params", "Pair", "Out", "RtsError", "params", "synth_pair", "gray_to_rgb", "rgb_to_lab",
           "HOST", "DEVICE", "COST_NONE", "COST_AD", "COST_RANK", "COST_CENSUS", "COST_LOG", "COST_NCC",
           "AGGR_NONE", "AGGR_BOX", "AGGR_AW", "AGGR_CROSS", "PREC_F32", "PREC_F16", "lib"]

LOG5x5 = np.array([0.0239, 0.046, 0.0499, 0.046, 0.0239,
                   0.046, 0.0061, -0.0923, 0.0061, 0.046,
                   0.0499, -0.0923, -0.3182, -0.0923, 0.0499,
                   0.046, 0.0061, -0.0923, 0.0061, 0.046,
                   0.0239, 0.046, 0.0499, 0.046, 0.0239], np.float32)  # seq/Main.cpp:113-117


def lib():
    return N.load()


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):  # torch tensor
        return a.data_ptr()
    raise TypeError(f"unsupported buffer type {type(a)}")


def params(**kw) -> Params:
    """rts_params with the reference driver's defaults (rts_params_default), overridden by kw."""
    p = Params()
    lib().rts_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def synth_pair(seed: int, width: int, height: int, max_disp: int, n_rects: int, n_planes: int = 0,
               sigma: float = 2.0, bg_disp: int = 4):
    """Seeded random-dot pair: (left_gray, right_gray, gt_disp)."""
    L = np.empty((height, width), np.uint8)
    R = np.empty((height, width), np.uint8)
    G = np.empty((height, width), np.uint8)
    st = lib().rts_synth_pair(seed, width, height, max_disp, n_rects, n_planes, sigma, bg_disp, _ptr(L), _ptr(R),
                              _ptr(G))
    if st != 0:
        raise RtsError(st, "rts_synth_pair")
    return L, R, G


def gray_to_rgb(g: np.ndarray) -> np.ndarray:
    H, W = g.shape
    out = np.empty((H, W, 3), np.uint8)
    lib().rts_gray_to_rgb(_ptr(np.ascontiguousarray(g)), _ptr(out), W, H)
    return out


def rgb_to_lab(rgb: np.ndarray) -> np.ndarray:
    H, W, _ = rgb.shape
    out = np.empty((H, W, 3), np.uint8)
    lib().rts_rgb_to_lab(_ptr(np.ascontiguousarray(rgb)), _ptr(out), W, H)
    return out


class Context:
    """An rts_ctx: one device, one stream, a scratch arena and an HBM budget."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self._lib = lib()
        h = C.c_void_p()
        st = self._lib.rts_ctx_create(C.byref(h), device, hbm_budget)
        if st != 0:
            raise RtsError(st, self._lib.rts_status_string(st).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self._lib.rts_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- plumbing ---------------------------------------------------------------
    def check(self, st: int, what: str = ""):
        if st != 0:
            msg = self._lib.rts_ctx_last_error(self.h).decode(errors="replace")
            raise RtsError(st, f"{what}: {msg}")

    def call(self, name: str, *args):
        """Call rts_<name>(ctx, *args) and raise on a non-OK status."""
        fn = getattr(self._lib, "rts_" + name)
        self.check(fn(self.h, *[_ptr(a) if isinstance(a, np.ndarray) or hasattr(a, "data_ptr") else a
                                for a in args]), name)

    def set_stream(self, stream_handle: int | None):
        self.check(self._lib.rts_ctx_set_stream(self.h, stream_handle), "set_stream")

    def synchronize(self):
        self.check(self._lib.rts_ctx_synchronize(self.h), "synchronize")

    @property
    def kernel_launches(self) -> int:
        return int(self._lib.rts_ctx_kernel_launches(self.h))

    def force_cross_tune(self, vert_rows: int = 0, grid_mult: int = 8, persistent: int = 0):
        """Fix the cross-based view kernels' tile (vert_rows 0: the autotuner's choice)."""
        self.check(self._lib.rts_ctx_force_cross_tune(self.h, vert_rows, grid_mult, persistent), "force_cross_tune")

    def tma_timeouts(self) -> int:
        """TMA tile copies on this device whose bounded wait gave up (0 in normal use)."""
        return int(self._lib.rts_ctx_tma_timeouts(self.h))

    @property
    def bytes_in_use(self) -> int:
        return int(self._lib.rts_ctx_bytes_in_use(self.h))

    def enable_stage_timing(self, on: bool = True):
        self.check(self._lib.rts_ctx_enable_stage_timing(self.h, 1 if on else 0), "stage timing")

    def stage_times(self) -> dict:
        n = 64
        names = (C.c_char_p * n)()
        launches = (C.c_uint64 * n)()
        ms = (C.c_double * n)()
        k = self._lib.rts_ctx_stage_times(self.h, names, launches, ms, n)
        return {names[j].decode(): (int(launches[j]), float(ms[j])) for j in range(min(k, n))}

    def reset_stage_times(self):
        self._lib.rts_ctx_reset_stage_times(self.h)

    # -- seq module API (HOST numpy arrays) ------------------------------------
    def pixelBasedL2R(self, ref, tar, D):
        H, W = ref.shape
        out = np.empty((H, W, D), np.float32)
        self.call("pixelBasedL2R", HOST, ref, tar, out, D, H, W)
        return out

    def pixelBasedR2L(self, ref, tar, D):
        H, W = ref.shape
        out = np.empty((H, W, D), np.float32)
        self.call("pixelBasedR2L", HOST, ref, tar, out, D, H, W)
        return out

    def pixelBasedCostL2R_Float(self, ref, tar, D):
        H, W = ref.shape
        out = np.empty((H, W, D), np.float32)
        self.call("pixelBasedCostL2R_Float", HOST, ref, tar, out, D, H, W)
        return out

    def pixelBasedCostR2L_Float(self, ref, tar, D):
        H, W = ref.shape
        out = np.empty((H, W, D), np.float32)
        self.call("pixelBasedCostR2L_Float", HOST, ref, tar, out, D, H, W)
        return out

    def pixelBasedCostL2R_Color(self, ref, tar, D, normOrNot=0, trunc=None):
        H, W, _ = ref.shape
        out = np.empty((H, W, D), np.float32)
        if trunc is None:
            self.call("pixelBasedCostL2R_Color", HOST, ref, tar, out, D, H, W, normOrNot)
        else:
            self.call("pixelBasedCostL2R_Color_trunc", HOST, ref, tar, out, D, H, W, C.c_float(trunc), normOrNot)
        return out

    def pixelBasedR2L_Color(self, ref, tar, D, normOrNot=0, trunc=None):
        H, W, _ = ref.shape
        out = np.empty((H, W, D), np.float32)
        if trunc is None:
            self.call("pixelBasedR2L_Color", HOST, ref, tar, out, D, H, W, normOrNot)
        else:
            self.call("pixelBasedR2L_Color_trunc", HOST, ref, tar, out, D, H, W, C.c_float(trunc), normOrNot)
        return out

    def calcCensusTrans(self, img, maskHrad=4, maskWrad=3):
        H, W = img.shape
        out = np.empty((H, W, (2 * maskHrad + 1) * (2 * maskWrad + 1)), np.uint8)
        self.call("calcCensusTrans", HOST, img, out, maskHrad, maskWrad, H, W)
        return out

    def calcHammingDist(self, bref, btar, D, maskHrad=4, maskWrad=3):
        H, W, _ = bref.shape
        out = np.empty((H, W, D), np.float32)
        self.call("calcHammingDist", HOST, bref, btar, out, maskHrad, maskWrad, H, W, D)
        return out

    def calculateRankFilt(self, img, maskSize):
        H, W = img.shape
        out = np.empty((H, W), np.uint8)
        self.call("calculateRankFilt", HOST, img, out, maskSize, H, W)
        return out

    def convolveImage(self, img, mask=LOG5x5, maskHrad=2, maskWrad=2):
        H, W = img.shape
        out = np.empty((H, W), np.float32)
        self.call("convolveImage", HOST, img, out, np.ascontiguousarray(mask, np.float32), H, W, maskHrad, maskWrad)
        return out

    def calcNCCDispL2R(self, ref, tar, D, maskHrad, maskWrad, fill=0.0):
        H, W = ref.shape
        out = np.full((H, W, D), fill, np.float32)
        self.call("calcNCCDispL2R", HOST, ref, tar, out, D, H, W, maskHrad, maskWrad)
        return out

    def combineCost(self, c1, c2, lambda1, lambda2):
        H, W, D = c1.shape
        out = np.array(c1, np.float32, copy=True)
        self.call("combineCost", HOST, out, np.ascontiguousarray(c2), C.c_float(lambda1), C.c_float(lambda2), H, W, D)
        return out

    def boxAggregate(self, cost, wndwRad):
        H, W, D = cost.shape
        out = np.array(cost, np.float32, copy=True)
        self.call("boxAggregate", HOST, out, H, W, D, wndwRad)
        return out

    def findCross(self, rgb, arm_len=17, tau=20):
        H, W, _ = rgb.shape
        horz = np.empty((H, W, 2), np.int32)
        vert = np.empty((H, W, 2), np.int32)
        self.call("findCross_ex", HOST, rgb, horz, vert, H, W, arm_len, tau)
        return horz, vert

    def aggregate_cost_horizontal(self, cost):
        H, W, D = cost.shape
        out = np.array(cost, np.float32, copy=True)
        self.call("aggregate_cost_horizontal", HOST, out, H, W, D)
        return out

    def cross_stereo_aggregation(self, pre, hr, ht, vr, vt):
        H, W, D = pre.shape
        out = np.empty_like(pre)
        self.call("cross_stereo_aggregation", HOST, pre, out, hr, ht, vr, vt, H, W, D)
        return out

    def disp_refinement(self, disp, horz, vert, D):
        H, W = disp.shape
        out = np.array(disp, np.uint8, copy=True)
        self.call("disp_refinement", HOST, out, horz, vert, H, W, D)
        return out

    def medianFilt(self, img, maskSize=3):
        """Median pre-filter of an arm image ([H][W] or [H][W][3]); returns a copy."""
        H, W = img.shape[:2]
        ch = 1 if img.ndim == 2 else img.shape[2]
        out = np.array(img, np.uint8, copy=True)
        self.call("medianFilt", HOST, out, H, W, ch, maskSize)
        return out

    def calcProxWeight(self, gamma_proximity, maskRad):
        out = np.empty(((2 * maskRad + 1) ** 2,), np.float32)
        self.call("calcProxWeight", HOST, out, C.c_float(gamma_proximity), maskRad)
        return out

    def computeWeights(self, proxWeight, lab, gamma_similarity, maskRad):
        H, W, _ = lab.shape
        out = np.empty((H, W, (2 * maskRad + 1) ** 2), np.float32)
        self.call("computeWeights", HOST, out, proxWeight, lab, C.c_float(gamma_similarity), H, W, maskRad)
        return out

    def calcAWCostL2R(self, wref, wtar, cost, maskRad):
        H, W, D = cost.shape
        out = np.empty_like(cost)
        self.call("calcAWCostL2R", HOST, wref, wtar, cost, out, H, W, D, maskRad)
        return out

    def calcAWCostR2L(self, wref, wtar, cost, maskRad):
        H, W, D = cost.shape
        out = np.array(cost, np.float32, copy=True)
        self.call("calcAWCostR2L", HOST, wref, wtar, out, H, W, D, maskRad)
        return out

    def WTA(self, cost):
        H, W, D = cost.shape
        out = np.empty((H, W), np.uint8)
        self.call("WTA", HOST, np.ascontiguousarray(cost), out, H, W, D)
        return out

    def WTA_NCC(self, cost):
        H, W, D = cost.shape
        out = np.empty((H, W), np.uint8)
        self.call("WTA_NCC", HOST, np.ascontiguousarray(cost), out, H, W, D)
        return out

    def cross_check(self, dref, dtar):
        H, W = dref.shape
        out = np.empty((H, W), np.uint8)
        self.call("cross_check", HOST, dref, dtar, out, H, W)
        return out

    # -- whole pipeline ----------------------------------------------------------
    def pipeline(self, p: Params, lgray, rgray, lrgb=None, rrgb=None, llab=None, rlab=None, want_cost=False):
        """HOST pipeline run; returns (disp_left, disp_right, mask, cost_left or None)."""
        H, W = lgray.shape
        pair = Pair(W, H, _ptr(lgray), _ptr(rgray), _ptr(lrgb), _ptr(rrgb), _ptr(llab), _ptr(rlab))
        dl = np.zeros((H, W), np.uint8)
        dr = np.zeros((H, W), np.uint8)
        mk = np.zeros((H, W), np.uint8)
        cost = np.empty((H, W, p.disp_range), np.float32) if want_cost else None
        out = Out(_ptr(dl), _ptr(dr), _ptr(mk), _ptr(cost))
        self.check(self._lib.rts_pipeline_run(self.h, HOST, C.byref(pair), C.byref(p), C.byref(out)), "pipeline")
        return dl, dr, mk, cost

    # -- batched form (DEVICE buffers) ---------------------------------------------
    def batch_run(self, pairs, params, outs):
        """rts_batch_run over lists of Pair / Params / Out holding DEVICE pointers."""
        n = len(pairs)
        PA, PR, PO = (Pair * n)(*pairs), (Params * n)(*params), (Out * n)(*outs)
        self.check(self._lib.rts_batch_run(self.h, n, PA, PR, PO), "batch_run")


class Server:
    """rts_server: continuous-batching request loop over one context."""

    def __init__(self, ctx: Context, hbm_budget: int, max_inflight: int = 64, max_batch: int = 16,
                 precision: int = PREC_F16, priority_pixels: int = 0):
        self.ctx = ctx
        self._lib = ctx._lib
        h = C.c_void_p()
        cfg = ServerConfig(hbm_budget, max_inflight, max_batch, precision, priority_pixels)
        ctx.check(self._lib.rts_server_create(C.byref(h), ctx.h, C.byref(cfg)), "server_create")
        self.h = h
        self._keep = {}

    def close(self):
        if getattr(self, "h", None):
            self._lib.rts_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, p: Params, lgray, rgray, lrgb=None, rrgb=None, outs=None):
        """Queues a pair (HOST arrays, copied now); returns (ticket, (disp_l, disp_r, mask)).
        outs: optional three [H][W] u8 arrays to receive the results (pinned ones are
        written by the device directly)."""
        H, W = lgray.shape
        pair = Pair(W, H, _ptr(lgray), _ptr(rgray), _ptr(lrgb), _ptr(rrgb), None, None)
        if outs is None:
            outs = tuple(np.zeros((H, W), np.uint8) for _ in range(3))
        out = Out(_ptr(outs[0]), _ptr(outs[1]), _ptr(outs[2]), None)
        t = C.c_uint64()
        st = self._lib.rts_server_submit(self.h, C.byref(pair), C.byref(p), C.byref(out), C.byref(t))
        if st != 0:
            raise RtsError(st, self._lib.rts_ctx_last_error(self.ctx.h).decode(errors="replace"))
        self._keep[t.value] = outs
        return t.value, outs

    def progress(self):
        self.ctx.check(self._lib.rts_server_progress(self.h), "server_progress")

    def poll(self, ticket) -> int:
        return int(self._lib.rts_server_poll(self.h, ticket))

    def cancel(self, ticket) -> int:
        return int(self._lib.rts_server_cancel(self.h, ticket))

    def tracked(self) -> int:
        """Requests the server still holds (pending, running, or not yet waited for)."""
        return int(self._lib.rts_server_tracked(self.h))

    def wait(self, ticket, timeout_ms: float = 60000.0):
        """Blocks until done; returns (submit_ms, start_ms, done_ms)."""
        st = RequestStats()
        r = self._lib.rts_server_wait(self.h, ticket, timeout_ms, C.byref(st))
        self._keep.pop(ticket, None)
        if r != 0:
            raise RtsError(r, "server_wait")
        return st.submit_ms, st.start_ms, st.done_ms
