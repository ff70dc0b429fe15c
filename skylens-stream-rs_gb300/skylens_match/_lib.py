"""ctypes bindings of libslm's C ABI (include/slm.h).

The library is the product: every matching call below runs the sm_103a
kernels. There is no CPU fallback; a missing library or device raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import buildlib as _build

P = ctypes.POINTER
c_u32, c_u64, c_f32, c_int = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float, ctypes.c_int

(SLM_OK, SLM_INVALID_ARG, SLM_CAPACITY, SLM_OOM, SLM_CUDA_ERROR, SLM_TIMEOUT, SLM_NO_DEVICE, SLM_INTERNAL,
 SLM_CANCELLED) = range(9)
PRECISIONS = {"fp32": 0, "bf16": 1, "fp8": 2, "auto": 3}  # auto: BF16 from 8M distances per call or batch


class SlmPair(ctypes.Structure):
    _fields_ = [("i", c_u32), ("j", c_u32)]


class SlmStats(ctypes.Structure):
    _fields_ = [("pairs", c_u64), ("distances", c_u64), ("matches", c_u64), ("rows_recomputed", c_u64),
                ("cols_recomputed", c_u64), ("rows_rescored", c_u64), ("kernel_ms", c_f32),
                ("max_abs_err", c_f32), ("kernel_launches", c_u64), ("pass_ms", c_f32 * 2),
                ("pairs_routed", c_u64), ("pairs_rescued", c_u64), ("rows_rescued", c_u64)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["pass_ms"] = list(d["pass_ms"])
        return d


class SlmOpts(ctypes.Structure):
    _fields_ = [("device", c_int), ("stream", ctypes.c_void_p), ("hbm_budget", c_u64)]


class SlmPairSchedule(ctypes.Structure):
    _fields_ = [("temporal", c_u64), ("pow2_max", c_u64), ("spec", c_int), ("range", c_u64),
                ("right_min", c_u64), ("left_min", c_u64), ("max", c_u64), ("step", c_u64)]


class SlmTune(ctypes.Structure):
    _fields_ = [("items_per_sm", c_u32), ("shortlist_k", c_u32), ("use_graph", c_u32), ("variant", c_u32),
                ("row_tiles", c_u32), ("autotune", c_u32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class SlmServerOpts(ctypes.Structure):
    _fields_ = [("device", c_int), ("hbm_budget", c_u64), ("max_descs", c_u64), ("max_views", c_u32),
                ("slots", c_u32), ("max_batch_pairs", c_u32), ("tick_us", c_u32), ("ratio", c_f32),
                ("mutual", c_int), ("prec", c_int)]


class SlmServerStats(ctypes.Structure):
    _fields_ = [("submitted", c_u64), ("completed", c_u64), ("batches", c_u64), ("pairs", c_u64),
                ("matches", c_u64), ("max_batch_requests", c_u64), ("max_inflight", c_u64),
                ("bytes_in_use", c_u64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class SlmKeypoint(ctypes.Structure):
    _fields_ = [("x", c_f32), ("y", c_f32), ("sigma", c_f32), ("response", c_f32), ("angle", c_f32)]


class SlmDetectorConfig(ctypes.Structure):
    _fields_ = [("octaves", c_u32), ("scales", c_u32), ("sigma0", c_f32), ("contrast", c_f32),
                ("edge_ratio", c_f32), ("max_features", c_u32), ("upscale_below", c_u32),
                ("upscale_fill", ctypes.c_int32)]


class SlmPairMatches(ctypes.Structure):
    _fields_ = [("image_a", c_u32), ("image_b", c_u32), ("first", c_u64), ("count", c_u64)]


class SlmTrackStats(ctypes.Structure):
    _fields_ = [("edges", c_u64), ("invalid_matches", c_u64), ("conflicts", c_u64), ("too_short", c_u64),
                ("truncated", c_u64), ("tracks", c_u64)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class SlmError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str):
        self.status = status
        names = ["SLM_OK", "SLM_INVALID_ARG", "SLM_CAPACITY", "SLM_OOM", "SLM_CUDA_ERROR", "SLM_TIMEOUT",
                 "SLM_NO_DEVICE", "SLM_INTERNAL", "SLM_CANCELLED"]
        name = names[status] if 0 <= status < len(names) else str(status)
        super().__init__(f"{where}: {name}: {detail}")


# Every function the header declares, with its ctypes signature.
SIGNATURES = {
    "slm_status_str": (ctypes.c_char_p, [c_int]),
    "slm_last_error": (ctypes.c_char_p, []),
    "slm_selftest_wait_timeout": (c_int, [ctypes.c_void_p, c_u32]),
    "slm_ctx_set_coalescing": (c_int, [ctypes.c_void_p, c_u32, c_u32]),
    "slm_ctx_coalescing_stats": (c_int, [ctypes.c_void_p, P(c_u64), P(c_u64), P(c_u64)]),
    "slm_ctx_create": (c_int, [P(SlmOpts), P(ctypes.c_void_p)]),
    "slm_ctx_destroy": (c_int, [ctypes.c_void_p]),
    "slm_ctx_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "slm_ctx_bytes_in_use": (c_u64, [ctypes.c_void_p]),
    "slm_ratio_match": (c_int, [ctypes.c_void_p, P(c_f32), c_u32, P(c_f32), c_u32, c_f32, c_int, c_int,
                                P(SlmPair), c_u32, P(c_u32), P(SlmStats)]),
    "slm_ratio_match_device": (c_int, [ctypes.c_void_p, ctypes.c_void_p, c_u32, ctypes.c_void_p, c_u32, c_f32,
                                       c_int, c_int, ctypes.c_void_p, c_u32, ctypes.c_void_p]),
    "slm_ratio_match_device_noalloc": (c_int, [ctypes.c_void_p, c_u32, ctypes.c_void_p, c_u32, c_f32, c_int,
                                               ctypes.c_void_p, c_u32, ctypes.c_void_p, ctypes.c_void_p]),
    "slm_candidate_pairs": (c_int, [P(c_u64), c_u32, c_u64, c_u64, c_u64, P(SlmPair), c_u64, P(c_u64)]),
    "slm_pair_schedule_default": (SlmPairSchedule, []),
    "slm_pair_schedule_spec": (SlmPairSchedule, []),
    "slm_scheduled_pairs": (c_int, [P(c_u64), c_u32, P(SlmPairSchedule), P(SlmPair), c_u64, P(c_u64)]),
    "slm_store_create": (c_int, [ctypes.c_void_p, c_u64, c_u32, P(ctypes.c_void_p)]),
    "slm_store_destroy": (c_int, [ctypes.c_void_p]),
    "slm_store_add_view": (c_int, [ctypes.c_void_p, ctypes.c_void_p, c_u32, P(c_u32)]),
    "slm_store_add_views": (c_int, [ctypes.c_void_p, ctypes.c_void_p, P(c_u64), P(c_u32), c_u32, P(c_u32)]),
    "slm_store_clear": (c_int, [ctypes.c_void_p]),
    "slm_store_num_views": (c_u32, [ctypes.c_void_p]),
    "slm_plan_create": (c_int, [ctypes.c_void_p, ctypes.c_void_p, P(SlmPair), c_u32, c_f32, c_int, c_int,
                                P(SlmTune), P(ctypes.c_void_p)]),
    "slm_plan_destroy": (c_int, [ctypes.c_void_p]),
    "slm_plan_launch": (c_int, [ctypes.c_void_p]),
    "slm_plan_results": (c_int, [ctypes.c_void_p, P(SlmPair), c_u64, P(c_u64), P(SlmStats)]),
    "slm_plan_device_results": (c_int, [ctypes.c_void_p, P(ctypes.c_void_p), P(ctypes.c_void_p),
                                        P(ctypes.c_void_p)]),
    "slm_plan_bytes": (c_u64, [ctypes.c_void_p]),
    "slm_plan_debug_dump": (c_int, [ctypes.c_void_p, P(c_f32), c_u64]),
    "slm_server_create": (c_int, [P(SlmServerOpts), P(ctypes.c_void_p)]),
    "slm_server_destroy": (c_int, [ctypes.c_void_p]),
    "slm_server_submit": (c_int, [ctypes.c_void_p, ctypes.c_void_p, c_u32, P(SlmPair), c_u32, P(c_u32), P(c_u64)]),
    "slm_server_submit_ptr": (c_int, [ctypes.c_void_p, ctypes.c_void_p, c_u32, P(SlmPair), c_u32, P(c_u32),
                                      P(c_u64)]),
    "slm_server_wait": (c_int, [ctypes.c_void_p, c_u64, c_u32, P(SlmPair), c_u64, P(c_u64),
                                P(ctypes.c_double)]),
    "slm_server_stats_get": (c_int, [ctypes.c_void_p, P(SlmServerStats)]),
    "slm_server_cancel": (c_int, [ctypes.c_void_p, c_u64]),
    "slm_autotune": (c_int, [ctypes.c_void_p, ctypes.c_void_p, P(SlmPair), c_u32, c_f32, c_int, c_int, P(SlmTune),
                             P(c_f32)]),
    "slm_match_batch": (c_int, [ctypes.c_void_p, ctypes.c_void_p, P(SlmPair), c_u32, c_f32, c_int, c_int,
                                P(SlmPair), c_u64, P(c_u64), P(SlmStats)]),
    "slm_plan_set_min_matches": (c_int, [ctypes.c_void_p, c_u32]),
    "slm_match_pairs": (c_int, [ctypes.c_void_p, ctypes.c_void_p, P(c_u64), c_u32, P(SlmPairSchedule), c_f32, c_int,
                                c_int, c_u32, P(SlmPair), c_u64, P(c_u64), P(SlmPair), c_u64, P(c_u64),
                                P(SlmStats)]),
    "slm_sampson_score": (c_int, [ctypes.c_void_p, P(ctypes.c_double), P(c_u64), c_u32, P(ctypes.c_double),
                                  P(ctypes.c_double), P(c_u32), c_u32, P(c_u32), P(c_u64), P(c_u32), c_u64]),
    "slm_detector_config_default": (None, [P(SlmDetectorConfig)]),
    "slm_detect_and_describe": (c_int, [ctypes.c_void_p, ctypes.c_void_p, c_u32, c_u32, c_u32,
                                        P(SlmDetectorConfig), ctypes.c_void_p, ctypes.c_void_p, c_u64, P(c_u64)]),
    "slm_detect_and_describe_rgb8": (c_int, [ctypes.c_void_p, ctypes.c_void_p, c_u32, c_u32, c_u32,
                                             P(SlmDetectorConfig), ctypes.c_void_p, ctypes.c_void_p, c_u64,
                                             P(c_u64)]),
    "slm_describe": (c_int, [ctypes.c_void_p, ctypes.c_void_p, c_u32, c_u32, ctypes.c_void_p, c_u32,
                             ctypes.c_void_p]),
    "slm_build_tracks_drop": (c_int, [ctypes.c_void_p, P(c_u32), c_u32, P(SlmPairMatches), c_u32, P(SlmPair), c_u32,
                                      c_u64, P(c_u64), c_u64, P(SlmPair), c_u64, P(c_u64), P(c_u64),
                                      P(SlmTrackStats)]),
}

_lock = threading.Lock()
_lib = None


def library_path() -> str:
    """libslm.so to load: $SLM_LIB_PATH if set (a build placed elsewhere), else the in-tree build."""
    return os.environ.get("SLM_LIB_PATH") or _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libslm.so (building it first if it is missing) and bind the ABI."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            if not build_if_missing or path != _build.LIB:
                raise RuntimeError(f"libslm is not built: {path} missing")
            _build.build()
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return L


def check(status: int, where: str) -> None:
    if status != SLM_OK:
        detail = load().slm_last_error().decode(errors="replace")
        raise SlmError(status, where, detail)
