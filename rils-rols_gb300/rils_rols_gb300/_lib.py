"""ctypes binding of librils_rols_gb300.so: the C ABI of include/rils_rols_gb300.h
(device fitness path), include/rils_rols_host.h (host search driver) and
include/rils_rols_serve.h (serving loop).

The library is built in-tree by build.py.  Loading never falls back to
anything else: a missing or unloadable library raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "librils_rols_gb300.so"

RRG_OK, RRG_E_INVALID, RRG_E_CUDA, RRG_E_NO_DEVICE, RRG_E_TIMEOUT, RRG_E_TOO_LARGE, RRG_E_OOM, RRG_E_DEVICE_FAULT = range(8)
RRG_PLAIN_FP64, RRG_MIXED, RRG_MIXED_CERTIFIED = 0, 1, 2
RRG_UNTUNED, RRG_TUNED = 0, 1
RRG_F_NONFINITE, RRG_F_RANK_DEFICIENT, RRG_F_QR_FALLBACK, RRG_F_VERIFIED_FP64, RRG_F_TOO_LARGE = 1, 2, 4, 8, 16
RRG_MAX_TERMS = 64
RRG_TUNE_OFF, RRG_TUNE_ON = 0, 1
RRG_KNOB_EVAL_WAVES, RRG_KNOB_FAC_GROUP, RRG_KNOB_PAIR_UNIT, RRG_KNOB_FAC_STAGE = 1, 2, 3, 4

STATUS_NAMES = {0: "RRG_OK", 1: "RRG_E_INVALID", 2: "RRG_E_CUDA", 3: "RRG_E_NO_DEVICE", 4: "RRG_E_TIMEOUT",
                5: "RRG_E_TOO_LARGE", 6: "RRG_E_OOM", 7: "RRG_E_DEVICE_FAULT"}


class Cand(C.Structure):
    _fields_ = [("code_offset", C.c_int32), ("code_len", C.c_int32), ("first_factor", C.c_int32),
                ("n_factors", C.c_int32), ("mode", C.c_int32), ("coef_offset", C.c_int32),
                ("stack_need", C.c_int32), ("reserved", C.c_int32)]


class Factor(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("reserved", C.c_int32)]


class Batch(C.Structure):
    _fields_ = [("n_cand", C.c_int32), ("n_factors", C.c_int32), ("n_code", C.c_int32), ("n_consts", C.c_int32),
                ("cands", C.POINTER(Cand)), ("factors", C.POINTER(Factor)), ("code", C.POINTER(C.c_uint32)),
                ("consts", C.POINTER(C.c_double))]


class Result(C.Structure):
    _fields_ = [("loss", C.c_double), ("rmse", C.c_double), ("size", C.c_int32), ("rank", C.c_int32),
                ("flags", C.c_uint32), ("n_coef", C.c_int32)]


class Backend(C.Structure):
    _fields_ = [("self", C.c_void_p), ("dataset_create", C.c_void_p), ("eval", C.c_void_p),
                ("predict", C.c_void_p), ("dataset_destroy", C.c_void_p)]


class JobParams(C.Structure):
    _fields_ = [("classification", C.c_int32), ("max_fit_calls", C.c_int32), ("max_seconds", C.c_int32),
                ("complexity_penalty", C.c_double), ("max_complexity", C.c_int32), ("sample_size", C.c_double),
                ("random_state", C.c_int32), ("precision", C.c_int32)]


class JobInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("fit_calls", C.c_int32), ("queued_s", C.c_double), ("run_s", C.c_double),
                ("time_to_model_s", C.c_double), ("best_time", C.c_double), ("footprint_bytes", C.c_int64),
                ("device_rounds", C.c_int64), ("candidates", C.c_int64)]


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("done", C.c_int64), ("failed", C.c_int64), ("running", C.c_int64),
                ("queued", C.c_int64), ("p50_time_to_model_s", C.c_double), ("p99_time_to_model_s", C.c_double),
                ("mean_time_to_model_s", C.c_double), ("wall_s", C.c_double), ("candidates", C.c_int64),
                ("peak_running", C.c_int64)]


# Every symbol the headers declare (checked by the CPU test suite).
EXPORTS = [
    "rrg_abi_version", "rrg_last_error", "rrg_context_create", "rrg_context_destroy", "rrg_dataset_create",
    "rrg_dataset_create_rows",
    "rrg_dataset_destroy", "rrg_round_submit", "rrg_round_wait", "rrg_eval", "rrg_predict", "rrg_batch_validate", "rrg_dataset_rows",
    "rrg_dataset_cols", "rrg_last_round_launches", "rrg_last_round_stats", "rrg_context_stream",
    "rrg_context_set_timing", "rrg_last_round_timing", "rrg_last_round_bytes", "rrg_eval_plain_noalloc", "rrg_context_set_limits",
    "rrg_device_memory", "rrg_tune_set_mode", "rrg_tune_pin", "rrg_tune_reset", "rrg_tune_report",
    "rrg_context_set_mixed_min_rows", "rrg_context_set_async", "rrg_context_set_graph", "rrg_context_memory",
    "rrg_context_set_column_cache", "rrg_context_clear_column_cache",
    "rrh_create", "rrh_destroy", "rrh_set_backend", "rrh_set_precision", "rrh_set_graph", "rrh_set_column_cache",
    "rrh_fit", "rrh_predict",
    "rrh_model_string", "rrh_model_prefix", "rrh_best_time", "rrh_total_time", "rrh_fit_calls", "rrh_counter",
    "rrh_last_error", "rrh_candidates", "rrh_rewrite", "rrh_encode", "rrh_rebuild",
    "rrs_create", "rrs_destroy", "rrs_set_backend", "rrs_submit", "rrs_wait", "rrs_result", "rrs_stats_get",
    "rrs_last_error",
]

_lock = threading.Lock()
_lib = None


def _declare(lib):
    P = C.POINTER
    vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    dp, cp = P(C.c_double), C.c_char_p
    sig = {
        "rrg_abi_version": (i32, []),
        "rrg_last_error": (cp, []),
        "rrg_context_create": (i32, [i32, P(vp)]),
        "rrg_context_destroy": (i32, [vp]),
        "rrg_dataset_create": (i32, [vp, dp, dp, i64, i32, P(vp)]),
        "rrg_dataset_create_rows": (i32, [vp, dp, dp, i64, i32, P(vp)]),
        "rrg_dataset_destroy": (i32, [vp]),
        "rrg_round_submit": (i32, [vp, P(Batch), i32, P(Result), dp]),
        "rrg_round_wait": (i32, [vp, i32]),
        "rrg_eval": (i32, [vp, P(Batch), i32, P(Result), dp]),
        "rrg_predict": (i32, [vp, P(Batch), dp]),
        "rrg_batch_validate": (i32, [P(Batch), i32]),
        "rrg_dataset_rows": (i64, [vp]),
        "rrg_dataset_cols": (i32, [vp]),
        "rrg_last_round_launches": (i64, [vp]),
        "rrg_last_round_stats": (i32, [vp, P(C.c_int64), i32]),
        "rrg_context_stream": (vp, [vp]),
        "rrg_context_set_timing": (i32, [vp, i32]),
        "rrg_last_round_timing": (i32, [vp, dp, P(C.c_int64), i32]),
        "rrg_last_round_bytes": (i32, [vp, dp, i32]),
        "rrg_eval_plain_noalloc": (i32, [vp, i64, vp, i64, i32, P(Batch), vp, vp, vp]),
        "rrg_context_set_limits": (i32, [vp, i64, i64]),
        "rrg_device_memory": (i32, [i32, P(C.c_int64), P(C.c_int64)]),
        "rrg_context_set_mixed_min_rows": (i32, [vp, i64]),
        "rrg_context_set_async": (i32, [vp, i32]),
        "rrg_context_set_column_cache": (i32, [vp, i32]),
        "rrg_context_clear_column_cache": (i32, [vp]),
        "rrg_context_set_graph": (i32, [vp, i32]),
        "rrg_context_memory": (i64, [vp]),
        "rrg_tune_set_mode": (i32, [i32]),
        "rrg_tune_pin": (i32, [i32, i32, i32]),
        "rrg_tune_reset": (i32, []),
        "rrg_tune_report": (i64, [cp, i64]),
        "rrh_create": (vp, [i32, i32, i32, dbl, i32, dbl, i32, i32]),
        "rrh_destroy": (None, [vp]),
        "rrh_set_backend": (i32, [vp, P(Backend)]),
        "rrh_set_precision": (i32, [vp, i32]),
        "rrh_set_graph": (i32, [vp, i32]),
        "rrh_set_column_cache": (i32, [vp, i32]),
        "rrh_fit": (i32, [vp, dp, dp, i32, i32]),
        "rrh_predict": (i32, [vp, dp, i32, i32, dp]),
        "rrh_model_string": (i32, [vp, cp, i32]),
        "rrh_model_prefix": (i32, [vp, cp, i32]),
        "rrh_best_time": (dbl, [vp]),
        "rrh_total_time": (dbl, [vp]),
        "rrh_fit_calls": (i32, [vp]),
        "rrh_counter": (i64, [vp, i32]),
        "rrh_last_error": (cp, []),
        "rrh_candidates": (i32, [cp, i32, i32, i32, cp, i32]),
        "rrh_rewrite": (i32, [cp, i32, cp, i32]),
        "rrh_encode": (i32, [cp, i32, P(Batch)]),
        "rrh_rebuild": (i32, [cp, dp, i32, cp, i32]),
        "rrs_create": (vp, [i32, i64, i32]),
        "rrs_destroy": (None, [vp]),
        "rrs_set_backend": (i32, [vp, P(Backend)]),
        "rrs_submit": (i64, [vp, dp, dp, i32, i32, P(JobParams)]),
        "rrs_wait": (i32, [vp, i64, i32]),
        "rrs_result": (i32, [vp, i64, cp, i32, P(JobInfo)]),
        "rrs_stats_get": (i32, [vp, P(ServeStats)]),
        "rrs_last_error": (cp, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def load(build_if_missing: bool = True):
    """The loaded library.  Builds it in-tree when missing; raises if it cannot."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                if not build_if_missing:
                    raise RuntimeError(f"{LIB_PATH} is missing; run the in-tree build first")
                from . import build
                build.build()
            lib = C.CDLL(str(LIB_PATH))
            _declare(lib)
            _lib = lib
        return _lib


def last_error() -> str:
    return load().rrg_last_error().decode(errors="replace")


class RRGError(RuntimeError):
    def __init__(self, status: int, where: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {last_error()}")
        self.status = status


def check(status: int, where: str):
    if status != RRG_OK:
        raise RRGError(status, where)
