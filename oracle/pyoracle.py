"""ORACLE loader - test infrastructure only (tests/, __graft_entry__.smoke() and
the CPU-baseline leg of bench.py).  Builds oracle/rrg_oracle.c with the host C
compiler into oracle/_build/ and scores rrg_batch batches with it."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "rrg_oracle.c"
LIB = HERE / "_build" / "liboracle.so"
CFLAGS = ["-std=c99", "-O2", "-ffp-contract=off", "-fPIC", "-shared"]


def build(force: bool = False) -> Path:
    common = HERE.parent / "rils-rols_gb300" / "csrc" / "common"
    srcs = [SRC, HERE / "colpiv_qr.h", HERE.parent / "include" / "rils_rols_gb300.h", common / "rr_sum.h",
            common / "rr_math.h"]
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(p.stat().st_mtime for p in srcs):
        return LIB
    LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(["gcc", *CFLAGS, str(SRC), "-o", str(tmp), "-lm", "-lpthread"], check=True)
    os.replace(tmp, LIB)
    return LIB


# rrg_result of include/rils_rols_gb300.h
RESULT_DT = np.dtype([("loss", np.float64), ("rmse", np.float64), ("size", np.int32), ("rank", np.int32),
                      ("flags", np.uint32), ("n_coef", np.int32)])
TUNED = 1


def decode(res: np.ndarray, coefs: np.ndarray, batch) -> dict:
    out = {k: res[k].copy() for k in ("loss", "rmse", "size", "rank", "flags")}
    c = batch.cands
    lo = c["coef_offset"].astype(np.int64)
    hi = np.where(c["mode"] == TUNED, lo + c["n_factors"] + 1, lo)
    out["coefs"] = [coefs[a:b] for a, b in zip(lo.tolist(), hi.tolist())]
    return out


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        lib.oracle_dataset_create.restype = C.c_void_p
        lib.oracle_dataset_create.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int64,
                                              C.c_int32]
        lib.oracle_dataset_destroy.argtypes = [C.c_void_p]
        lib.oracle_eval_threads.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
        lib.oracle_eval_threads.restype = C.c_int32
        lib.oracle_predict.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
        lib.oracle_predict.restype = C.c_int32
        _lib = lib
    return _lib


class OracleDataset:
    def __init__(self, X: np.ndarray, y: np.ndarray):
        X = np.asarray(X, dtype=np.float64)
        if X.ndim == 1:
            X = X[:, None]
        self.n, self.d = X.shape
        self._X = np.ascontiguousarray(X.T)
        self._y = np.ascontiguousarray(np.asarray(y, dtype=np.float64))
        dp = C.POINTER(C.c_double)
        self.h = load().oracle_dataset_create(None, self._X.ctypes.data_as(dp), self._y.ctypes.data_as(dp), self.n,
                                              self.d)
        if not self.h:
            raise MemoryError("oracle dataset")

    def evaluate(self, batch, threads: int = 1) -> dict:
        """Per-candidate loss, rmse, size, rank, flags and coefficients (the
        fields of rils_rols_gb300.fitness.Dataset.evaluate).  `batch` is any
        object with the rrg_batch arrays (cands, n_coefs) and a struct()
        method: oracle.tree_encode.encode makes one without the product."""
        res = np.zeros(len(batch), dtype=RESULT_DT)
        coefs = np.zeros(max(1, batch.n_coefs), dtype=np.float64)
        b = batch.struct()
        st = load().oracle_eval_threads(self.h, C.addressof(b), res.ctypes.data, coefs.ctypes.data, threads)
        if st != 0:
            raise RuntimeError(f"oracle_eval failed with status {st}")
        return decode(res, coefs, batch)

    def predict(self, batch) -> np.ndarray:
        out = np.zeros(self.n)
        b = batch.struct()
        if load().oracle_predict(self.h, C.addressof(b), out.ctypes.data_as(C.POINTER(C.c_double))) != 0:
            raise RuntimeError("oracle_predict failed")
        return out

    def __del__(self):
        try:
            load().oracle_dataset_destroy(self.h)
        except Exception:
            pass


def backend_struct():
    """An rrh_backend (include/rils_rols_host.h) whose functions are the oracle's."""
    from rils_rols_gb300._lib import Backend
    lib = load()
    return Backend(None, C.cast(lib.oracle_dataset_create, C.c_void_p), C.cast(lib.oracle_eval, C.c_void_p),
                   C.cast(lib.oracle_predict, C.c_void_p), C.cast(lib.oracle_dataset_destroy, C.c_void_p))
