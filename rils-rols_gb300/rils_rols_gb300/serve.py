"""Serving loop over the device path (include/rils_rols_serve.h).

    srv = Server(max_active=4)
    job = srv.submit(X, y, max_fit_calls=100000, random_state=0)
    model, info = srv.result(job)          # waits for the model
    srv.stats()                            # p50 / p99 time to model, jobs, candidates

Each job is one fit of the reference's RILSROLSRegressor / RILSROLSBinaryClassifier
(rils_rols/rils_rols.py:9-76) run by the host search driver with its own device
context; the jobs in flight share the GPU, admitted in arrival order while
their device-memory footprints fit the budget.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import JobInfo, JobParams, ServeStats

STATES = {0: "queued", 1: "running", 2: "done", 3: "failed"}


class ServeError(RuntimeError):
    pass


class Server:
    def __init__(self, device: int = 0, memory_budget: int = 0, max_active: int = 4, backend=None):
        self._lib = _lib.load()
        self._h = self._lib.rrs_create(device, memory_budget, max_active)
        if not self._h:
            raise ServeError(self._lib.rrs_last_error().decode(errors="replace"))
        if backend is not None:
            self._backend = backend  # kept alive while the server uses its function pointers
            if self._lib.rrs_set_backend(self._h, C.byref(backend)) != _lib.RRG_OK:
                raise ServeError(self._lib.rrs_last_error().decode(errors="replace"))

    def close(self):
        if self._h:
            self._lib.rrs_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, X, y, *, classification=False, max_fit_calls=100000, max_seconds=100, complexity_penalty=0.001,
               max_complexity=50, sample_size=1.0, random_state=0, precision=_lib.RRG_PLAIN_FP64) -> int:
        """Queue one fit; the arguments are those of rils_rols(...) (rils_rols_cpp/rils_rols_cpp.cpp:646-657)."""
        X = np.ascontiguousarray(X, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1)
        if X.ndim != 2 or X.shape[0] != y.shape[0]:
            raise ValueError("X must be (n, d) with n == len(y)")
        p = JobParams(int(bool(classification)), int(max_fit_calls), int(max_seconds), float(complexity_penalty),
                      int(max_complexity), float(sample_size), int(random_state), int(precision))
        dp = C.POINTER(C.c_double)
        job = self._lib.rrs_submit(self._h, X.ctypes.data_as(dp), y.ctypes.data_as(dp), X.shape[0], X.shape[1],
                                   C.byref(p))
        if job < 0:
            raise ServeError(f"{_lib.STATUS_NAMES.get(-job, -job)}: "
                             f"{self._lib.rrs_last_error().decode(errors='replace')}")
        return int(job)

    def wait(self, job: int, timeout_ms: int = -1) -> bool:
        st = self._lib.rrs_wait(self._h, job, timeout_ms)
        if st == _lib.RRG_E_TIMEOUT:
            return False
        if st != _lib.RRG_OK:
            raise ServeError(self._lib.rrs_last_error().decode(errors="replace"))
        return True

    def info(self, job: int) -> dict:
        info = JobInfo()
        self._lib.rrs_result(self._h, job, None, 0, C.byref(info))
        return self._info_dict(info)

    def result(self, job: int, timeout_ms: int = -1):
        """(model string, info) of a finished job; raises ServeError for a failed one."""
        if not self.wait(job, timeout_ms):
            raise TimeoutError(f"job {job} has not finished")
        info = JobInfo()
        need = -self._lib.rrs_result(self._h, job, None, 0, C.byref(info))
        buf = C.create_string_buffer(max(need, 1))
        self._lib.rrs_result(self._h, job, buf, len(buf), C.byref(info))
        text = buf.value.decode()
        d = self._info_dict(info)
        if d["state"] == "failed":
            raise ServeError(f"job {job} failed: {text}")
        return text, d

    def stats(self) -> dict:
        s = ServeStats()
        self._lib.rrs_stats_get(self._h, C.byref(s))
        return {k: getattr(s, k) for k, _ in ServeStats._fields_}

    @staticmethod
    def _info_dict(info: JobInfo) -> dict:
        d = {k: getattr(info, k) for k, _ in JobInfo._fields_}
        d["state"] = STATES.get(d["state"], d["state"])
        return d
