"""ctypes binding of the C ABI declared in include/rtstereo.h.

The library is the in-tree ``librtstereo_gb300.so`` built by
``rtstereo_gb300/build.py``.  There is no fallback: if the library is missing
or cannot be loaded, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "librtstereo_gb300.so")

p, i, f, sz, u64, d = C.c_void_p, C.c_int, C.c_float, C.c_size_t, C.c_uint64, C.c_double

RTS_OK, RTS_ERR_INVALID_ARG, RTS_ERR_OOM, RTS_ERR_CUDA, RTS_ERR_TIMEOUT, RTS_ERR_UNSUPPORTED, \
    RTS_ERR_BUSY, RTS_ERR_CANCELLED = range(8)
HOST, DEVICE = 0, 1
COST_NONE, COST_AD, COST_RANK, COST_CENSUS, COST_LOG, COST_NCC = range(6)
AGGR_NONE, AGGR_BOX, AGGR_AW, AGGR_CROSS = range(4)
PREC_F32, PREC_F16 = 0, 1


class Params(C.Structure):
    """rts_params"""
    _fields_ = [("cost1", i), ("cost2", i), ("aggr", i), ("lambda1", f), ("lambda2", f), ("disp_range", i),
                ("census_hrad", i), ("census_wrad", i), ("rank_rad", i), ("ncc_hrad", i), ("ncc_wrad", i),
                ("box_rad", i), ("aw_rad", i), ("aw_gamma_s", f), ("aw_gamma_p", f), ("cross_arm", i),
                ("cross_tau", i), ("ad_trunc", f), ("right_view", i), ("precision", i),
                ("median_ksize", i)]


class Pair(C.Structure):
    """rts_pair"""
    _fields_ = [("width", i), ("height", i), ("left_gray", p), ("right_gray", p), ("left_rgb", p),
                ("right_rgb", p), ("left_lab", p), ("right_lab", p)]


class Out(C.Structure):
    """rts_out"""
    _fields_ = [("disp_left", p), ("disp_right", p), ("mask", p), ("cost_left", p)]


class ServerConfig(C.Structure):
    """rts_server_config"""
    _fields_ = [("hbm_budget", sz), ("max_inflight", i), ("max_batch", i), ("precision", i),
                ("priority_pixels", C.c_longlong)]


class RequestStats(C.Structure):
    """rts_request_stats"""
    _fields_ = [("submit_ms", d), ("start_ms", d), ("done_ms", d)]


PP = C.POINTER(p)

# symbol -> (restype, argtypes); every function declared in include/rtstereo.h
SIGNATURES = {
    "rts_ctx_create": (i, [PP, i, sz]),
    "rts_ctx_destroy": (None, [p]),
    "rts_ctx_set_stream": (i, [p, p]),
    "rts_ctx_stream": (p, [p]),
    "rts_ctx_synchronize": (i, [p]),
    "rts_ctx_bytes_in_use": (sz, [p]),
    "rts_ctx_last_error": (C.c_char_p, [p]),
    "rts_status_string": (C.c_char_p, [i]),
    "rts_ctx_kernel_launches": (u64, [p]),
    "rts_ctx_tma_timeouts": (u64, [p]),
    "rts_ctx_force_cross_tune": (i, [p, i, i, i]),
    "rts_ctx_enable_stage_timing": (i, [p, i]),
    "rts_ctx_stage_times": (i, [p, C.POINTER(C.c_char_p), C.POINTER(u64), C.POINTER(d), i]),
    "rts_ctx_reset_stage_times": (None, [p]),
    "rts_pixelBasedL2R": (i, [p, i, p, p, p, i, i, i]),
    "rts_pixelBasedR2L": (i, [p, i, p, p, p, i, i, i]),
    "rts_pixelBasedCostL2R_Float": (i, [p, i, p, p, p, i, i, i]),
    "rts_pixelBasedCostR2L_Float": (i, [p, i, p, p, p, i, i, i]),
    "rts_pixelBasedCostL2R_Color": (i, [p, i, p, p, p, i, i, i, i]),
    "rts_pixelBasedCostL2R_Color_trunc": (i, [p, i, p, p, p, i, i, i, f, i]),
    "rts_pixelBasedR2L_Color": (i, [p, i, p, p, p, i, i, i, i]),
    "rts_pixelBasedR2L_Color_trunc": (i, [p, i, p, p, p, i, i, i, f, i]),
    "rts_calcCensusTrans": (i, [p, i, p, p, i, i, i, i]),
    "rts_calcHammingDist": (i, [p, i, p, p, p, i, i, i, i, i]),
    "rts_calculateRankFilt": (i, [p, i, p, p, i, i, i]),
    "rts_convolveImage": (i, [p, i, p, p, p, i, i, i, i]),
    "rts_calcNCCDispL2R": (i, [p, i, p, p, p, i, i, i, i, i]),
    "rts_combineCost": (i, [p, i, p, p, f, f, i, i, i]),
    "rts_boxAggregate": (i, [p, i, p, i, i, i, i]),
    "rts_findCross": (i, [p, i, p, p, p, i, i]),
    "rts_findCross_ex": (i, [p, i, p, p, p, i, i, i, i]),
    "rts_aggregate_cost_horizontal": (i, [p, i, p, i, i, i]),
    "rts_cross_stereo_aggregation": (i, [p, i, p, p, p, p, p, p, i, i, i]),
    "rts_disp_refinement": (i, [p, i, p, p, p, i, i, i]),
    "rts_medianFilt": (i, [p, i, p, i, i, i, i]),
    "rts_calcProxWeight": (i, [p, i, p, f, i]),
    "rts_computeWeights": (i, [p, i, p, p, p, f, i, i, i]),
    "rts_calcAWCostL2R": (i, [p, i, p, p, p, p, i, i, i, i]),
    "rts_calcAWCostR2L": (i, [p, i, p, p, p, i, i, i, i]),
    "rts_WTA": (i, [p, i, p, p, i, i, i]),
    "rts_WTA_NCC": (i, [p, i, p, p, i, i, i]),
    "rts_cross_check": (i, [p, i, p, p, p, i, i]),
    "rts_WTA_noalloc": (i, [p, p, i, i, i, p]),
    "rts_params_default": (None, [C.POINTER(Params)]),
    "rts_pipeline_run": (i, [p, i, C.POINTER(Pair), C.POINTER(Params), C.POINTER(Out)]),
    "rts_batch_run": (i, [p, i, C.POINTER(Pair), C.POINTER(Params), C.POINTER(Out)]),
    "rts_server_create": (i, [PP, p, C.POINTER(ServerConfig)]),
    "rts_server_destroy": (None, [p]),
    "rts_server_submit": (i, [p, C.POINTER(Pair), C.POINTER(Params), C.POINTER(Out), C.POINTER(u64)]),
    "rts_server_poll": (i, [p, u64]),
    "rts_server_wait": (i, [p, u64, d, C.POINTER(RequestStats)]),
    "rts_server_cancel": (i, [p, u64]),
    "rts_server_progress": (i, [p]),
    "rts_server_tracked": (C.c_long, [p]),
    "rts_synth_pair": (i, [u64, i, i, i, i, i, f, i, p, p, p]),
    "rts_gray_to_rgb": (None, [p, p, i, i]),
    "rts_rgb_to_lab": (None, [p, p, i, i]),
}

_LIB = None


def load(build_if_missing: bool = False):
    """Load the native library (building it first if asked and absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build as _b
            _b.build()
        else:
            raise RuntimeError(
                f"rtstereo_gb300 native library not found at {LIB_PATH}; run "
                "`python -c 'import __graft_entry__ as g; g.build()'` (or python rtstereo_gb300/build.py)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class RtsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"rtstereo status {status}: {msg}")
        self.status = status
