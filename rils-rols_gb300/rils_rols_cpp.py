"""Drop-in for the reference's pybind11 module `rils_rols_cpp`
(rils_rols_cpp/rils_rols_cpp.cpp:998-1007): class `rils_rols` with the same
constructor, fit / predict and getters, backed by the host search driver of
librils_rols_gb300.so whose fitness runs on the GB300 device path.

Differences that a caller can see: bad input raises ValueError / RuntimeError
instead of exiting the process (rils_rols_cpp.cpp:722-725, 733-736).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from rils_rols_gb300 import _lib
from rils_rols_gb300._lib import RRG_MIXED, RRG_MIXED_CERTIFIED, RRG_PLAIN_FP64


class rils_rols:  # noqa: N801 - name of the reference class
    def __init__(self, classification: bool, max_fit_calls: int, max_seconds: int, complexity_penalty: float,
                 max_complexity: int, sample_size: float, verbose: bool, random_state: int):
        self._lib = _lib.load()
        self._h = self._lib.rrh_create(int(bool(classification)), int(max_fit_calls), int(max_seconds),
                                       float(complexity_penalty), int(max_complexity), float(sample_size),
                                       int(bool(verbose)), int(random_state))
        if not self._h:
            raise RuntimeError(self._lib.rrh_last_error().decode())
        self._backend = None

    # -- extensions beyond the reference's module --
    def set_backend(self, backend) -> None:
        """Install an rrh_backend struct (None restores the GB300 device path)."""
        self._backend = backend
        _lib.check(self._lib.rrh_set_backend(self._h, C.byref(backend) if backend is not None else None),
                   "rrh_set_backend")

    def set_precision(self, precision: str | int) -> None:
        p = {"plain": RRG_PLAIN_FP64, "fp64": RRG_PLAIN_FP64, "mixed": RRG_MIXED_CERTIFIED,
             "mixed_uncertified": RRG_MIXED}.get(precision, precision)
        _lib.check(self._lib.rrh_set_precision(self._h, int(p)), "rrh_set_precision")

    def set_graph(self, on: bool = True) -> None:
        """Run the device rounds as CUDA graphs (the same search and results)."""
        _lib.check(self._lib.rrh_set_graph(self._h, int(bool(on))), "rrh_set_graph")

    def set_column_cache(self, on: bool = True) -> None:
        """Keep factor columns across the device rounds (on by default; the same
        search and results)."""
        _lib.check(self._lib.rrh_set_column_cache(self._h, int(bool(on))), "rrh_set_column_cache")

    def counters(self) -> dict:
        names = ["ls_calls", "main_it", "device_rounds", "candidates_scored", "skipped_perts", "total_perts",
                 "backend_ns"]
        return {n: int(self._lib.rrh_counter(self._h, i)) for i, n in enumerate(names)}

    def get_model_prefix(self) -> str:
        return self._text(self._lib.rrh_model_prefix)

    # -- the reference's interface --
    def fit(self, X, y, data_cnt: int, feat_cnt: int) -> None:
        Xa = np.ascontiguousarray(np.asarray(X, dtype=np.float64).reshape(-1))
        ya = np.ascontiguousarray(np.asarray(y, dtype=np.float64).reshape(-1))
        if Xa.size != data_cnt * feat_cnt:
            raise ValueError(f"Size of X {Xa.size} is not the same as the product of data count and feature count "
                             f"{data_cnt * feat_cnt}")
        if ya.size != data_cnt:
            raise ValueError(f"Size of y {ya.size} is not the same as the data count {data_cnt}")
        dp = C.POINTER(C.c_double)
        st = self._lib.rrh_fit(self._h, Xa.ctypes.data_as(dp), ya.ctypes.data_as(dp), int(data_cnt), int(feat_cnt))
        if st != 0:
            raise RuntimeError(f"fit failed: {_lib.STATUS_NAMES.get(st, st)}: {self._lib.rrh_last_error().decode()}")

    def predict(self, X, data_cnt: int, feat_cnt: int) -> np.ndarray:
        Xa = np.ascontiguousarray(np.asarray(X, dtype=np.float64).reshape(-1))
        if Xa.size != data_cnt * feat_cnt:
            raise ValueError(f"Size of X {Xa.size} is not the same as the product of data count and feature count "
                             f"{data_cnt * feat_cnt}")
        out = np.zeros(int(data_cnt), dtype=np.float64)
        dp = C.POINTER(C.c_double)
        st = self._lib.rrh_predict(self._h, Xa.ctypes.data_as(dp), int(data_cnt), int(feat_cnt), out.ctypes.data_as(dp))
        if st != 0:
            raise RuntimeError(f"predict failed: {_lib.STATUS_NAMES.get(st, st)}: {self._lib.rrh_last_error().decode()}")
        return out

    def _text(self, fn) -> str:
        buf = C.create_string_buffer(1 << 16)
        r = fn(self._h, buf, len(buf))
        if r < 0:
            buf = C.create_string_buffer(-r + 16)
            r = fn(self._h, buf, len(buf))
        return buf.value.decode()

    def get_model_string(self) -> str:
        return self._text(self._lib.rrh_model_string)

    def get_best_time(self) -> float:
        return float(self._lib.rrh_best_time(self._h))

    def get_fit_calls(self) -> int:
        return int(self._lib.rrh_fit_calls(self._h))

    def get_total_time(self) -> float:
        return float(self._lib.rrh_total_time(self._h))

    def __del__(self):
        try:
            if self._h:
                self._lib.rrh_destroy(self._h)
                self._h = None
        except Exception:
            pass
