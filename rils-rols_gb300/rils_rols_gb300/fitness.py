"""Python view of the batched fitness C ABI (include/rils_rols_gb300.h).

    ctx = Context()                       # one CUDA stream + scratch on device 0
    ds = ctx.dataset(X, y)                # X: n x d (row-major) float64, resident in HBM
    batch = encode(trees, tuned=True)     # trees in prefix form, e.g. "add x0 mul c:2 sin x1"
    out = ds.evaluate(batch, precision=MIXED)

`out` holds per-candidate loss (1 - R2), rmse, size, rank, flags and the
fitted coefficients (free term last), exactly what the reference's
tune_constants + fitness return per candidate (rils_rols_cpp.cpp:445-541).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import RRG_MIXED, RRG_MIXED_CERTIFIED, RRG_PLAIN_FP64, RRG_TUNED, RRG_UNTUNED, Batch, Cand, Factor, Result, check

PLAIN = RRG_PLAIN_FP64
MIXED = RRG_MIXED
CERTIFIED = RRG_MIXED_CERTIFIED


@dataclass
class EncodedBatch:
    """An rrg_batch whose arrays are owned by numpy."""
    cands: np.ndarray
    factors: np.ndarray
    code: np.ndarray
    consts: np.ndarray
    n_coefs: int

    def __len__(self) -> int:
        return len(self.cands)

    def struct(self) -> Batch:
        b = Batch()
        b.n_cand = len(self.cands)
        b.n_factors = len(self.factors)
        b.n_code = len(self.code)
        b.n_consts = len(self.consts)
        b.cands = self.cands.ctypes.data_as(C.POINTER(Cand))
        b.factors = self.factors.ctypes.data_as(C.POINTER(Factor))
        b.code = self.code.ctypes.data_as(C.POINTER(C.c_uint32))
        b.consts = self.consts.ctypes.data_as(C.POINTER(C.c_double))
        return b


_CAND_DT = np.dtype([(n, np.int32) for n, _ in Cand._fields_])
_FACT_DT = np.dtype([(n, np.int32) for n, _ in Factor._fields_])
_RES_DT = np.dtype([("loss", np.float64), ("rmse", np.float64), ("size", np.int32), ("rank", np.int32),
                    ("flags", np.uint32), ("n_coef", np.int32)])


def encode(trees: list[str], tuned: bool = True) -> EncodedBatch:
    """Flatten prefix-form trees into postfix programs (host library, rrh_encode).

    tuned=True splits each tree into its top-level factors as tune_constants
    does (rils_rols_cpp.cpp:448-475); tuned=False scores the tree as given.
    """
    lib = _lib.load()
    b = Batch()
    text = "\n".join(trees).encode()
    check(lib.rrh_encode(text, RRG_TUNED if tuned else RRG_UNTUNED, C.byref(b)), "rrh_encode")
    def arr(ptr, n, dt):
        if n == 0:
            return np.zeros(0, dtype=dt)
        raw = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_byte)), shape=(n * np.dtype(dt).itemsize,))
        return raw.view(dt).copy()
    cands = arr(b.cands, b.n_cand, _CAND_DT)
    factors = arr(b.factors, b.n_factors, _FACT_DT)
    code = arr(b.code, b.n_code, np.uint32)
    consts = arr(b.consts, b.n_consts, np.float64)
    n_coefs = int(np.max(cands["coef_offset"] + cands["n_factors"] + 1)) if tuned and len(cands) else 0
    return EncodedBatch(cands, factors, code, consts, n_coefs)


def candidates(tree: str, d: int, local_search: bool = True, classification: bool = False) -> list[str]:
    """The candidates one search step generates from `tree` (all_candidates of
    rils_rols_cpp.cpp:348-443), in prefix form, in the reference's order."""
    lib = _lib.load()
    cap = 1 << 22
    while True:
        buf = C.create_string_buffer(cap)
        r = lib.rrh_candidates(tree.encode(), int(local_search), int(d), int(classification), buf, cap)
        if r >= 0:
            break
        if r == -1 or -r <= cap:
            raise _lib.RRGError(_lib.RRG_E_INVALID, "rrh_candidates")
        cap = -r + 16
    return [line.split("\t")[1] for line in buf.value.decode().split("\n") if line]


def decode_results(res: np.ndarray, coefs: np.ndarray, batch: EncodedBatch) -> dict:
    """Per-candidate fields, and each candidate's coefficients as a view into
    `coefs` (free term last; empty for untuned candidates)."""
    out = {k: res[k].copy() for k in ("loss", "rmse", "size", "rank", "flags")}
    c = batch.cands
    lo = c["coef_offset"].astype(np.int64)
    hi = np.where(c["mode"] == RRG_TUNED, lo + c["n_factors"] + 1, lo)
    out["coefs"] = [coefs[a:b] for a, b in zip(lo.tolist(), hi.tolist())]
    return out


class Context:
    """rrg_context on one device (default 0)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.rrg_context_create(device, C.byref(h)), "rrg_context_create")
        self.h = h

    def dataset(self, X: np.ndarray, y: np.ndarray) -> "Dataset":
        return Dataset(self, X, y)

    def last_round_launches(self) -> int:
        return int(self.lib.rrg_last_round_launches(self.h))

    REASONS = ("probe_nonfinite", "fp64_inf", "fp32_overflow", "nan_rank", "rank", "ill_cond", "snap", "drop",
               "one_pass", "cert", "other_nan")

    def last_round_stats(self) -> dict:
        out = (C.c_int64 * 25)()
        self.lib.rrg_last_round_stats(self.h, out, 25)
        d = {"launches": out[0], "plain_routed": out[1], "fp64_rescored": out[2], "residual_pass": out[3],
             "qr_skipped_sentinel": out[15], "distinct": out[16], "tiled_qr": bool(out[17]), "graph": bool(out[18]),
             "cache_hits": out[19], "cache_evals": out[20], "cache64_hits": out[21], "cache64_evals": out[22],
             "pair_hits": out[23], "pair_evals": out[24]}
        d["rescore_reasons"] = {r: out[4 + i] for i, r in enumerate(self.REASONS) if out[4 + i]}
        return d

    PHASES = ("factor_eval", "mixed_solve", "mixed_residual", "finalize", "fp64_eval", "fp64_qr", "fp64_residual",
              "pair_sums")

    def set_timing(self, on: bool = True) -> None:
        check(self.lib.rrg_context_set_timing(self.h, int(on)), "rrg_context_set_timing")

    def set_mixed_min_rows(self, rows: int) -> None:
        """Datasets with fewer rows run mixed-precision rounds in FP64 (default
        8192; 0 always takes the mixed form)."""
        check(self.lib.rrg_context_set_mixed_min_rows(self.h, int(rows)), "rrg_context_set_mixed_min_rows")

    def set_async(self, on: bool = True) -> None:
        """Mixed rounds decide their second half on the device (on, the
        default) or read their flags back to the host twice (off); the same
        results either way."""
        check(self.lib.rrg_context_set_async(self.h, int(on)), "rrg_context_set_async")

    def set_limits(self, scratch_bytes: int, table_bytes: int) -> None:
        """Device-memory limits of the FP64 tables and QR working columns
        (scratch) and of the double-float factor table (each >= 1 MiB)."""
        check(self.lib.rrg_context_set_limits(self.h, int(scratch_bytes), int(table_bytes)), "rrg_context_set_limits")

    def memory(self) -> int:
        """Device bytes the context's buffers hold (tables, column caches,
        scratch; datasets not included)."""
        return int(self.lib.rrg_context_memory(self.h))

    def set_column_cache(self, on: bool = True) -> None:
        """Keep factor columns on the device across rounds of one dataset (on,
        the default); the same results either way."""
        check(self.lib.rrg_context_set_column_cache(self.h, int(on)), "rrg_context_set_column_cache")

    def clear_column_cache(self) -> None:
        """Forget every kept column: the next round evaluates all its factors."""
        check(self.lib.rrg_context_clear_column_cache(self.h), "rrg_context_clear_column_cache")

    def set_graph(self, on: bool = True) -> None:
        """Run every round as a CUDA graph (rounds that cannot be captured are
        launched directly); the same results either way."""
        check(self.lib.rrg_context_set_graph(self.h, int(on)), "rrg_context_set_graph")

    def last_round_timing(self) -> dict:
        n = len(self.PHASES)
        ms = (C.c_double * n)()
        cnt = (C.c_int64 * n)()
        self.lib.rrg_last_round_timing(self.h, ms, cnt, n)
        return {p: (ms[i], cnt[i]) for i, p in enumerate(self.PHASES)}

    def last_round_bytes(self) -> dict:
        """Algorithmic device-memory bytes of the last round per phase (0 where not counted)."""
        n = len(self.PHASES)
        b = (C.c_double * n)()
        self.lib.rrg_last_round_bytes(self.h, b, n)
        return {p: b[i] for i, p in enumerate(self.PHASES)}

    def stream(self) -> int:
        """cudaStream_t of this context, as an integer handle."""
        return int(self.lib.rrg_context_stream(self.h) or 0)

    def close(self):
        if self.h:
            self.lib.rrg_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Dataset:
    """rrg_dataset: X (n x d, any layout) and y made resident on the device."""

    def __init__(self, ctx: Context, X: np.ndarray, y: np.ndarray):
        self.ctx = ctx
        X = np.asarray(X, dtype=np.float64)
        if X.ndim == 1:
            X = X[:, None]
        self.n, self.d = X.shape
        yv = np.ascontiguousarray(np.asarray(y, dtype=np.float64).reshape(-1))
        if len(yv) != self.n:
            raise ValueError("X and y disagree on the number of rows")
        h = C.c_void_p()
        dp = C.POINTER(C.c_double)
        if X.flags.f_contiguous and not X.flags.c_contiguous:
            # columns already contiguous
            check(ctx.lib.rrg_dataset_create(ctx.h, X.ctypes.data_as(dp), yv.ctypes.data_as(dp), self.n, self.d,
                                             C.byref(h)), "rrg_dataset_create")
        else:
            # rows as given (the device transposes)
            Xr = np.ascontiguousarray(X)
            check(ctx.lib.rrg_dataset_create_rows(ctx.h, Xr.ctypes.data_as(dp), yv.ctypes.data_as(dp), self.n,
                                                  self.d, C.byref(h)), "rrg_dataset_create_rows")
        self.h = h

    def evaluate(self, batch: EncodedBatch, precision: int = PLAIN) -> dict:
        res = np.zeros(len(batch), dtype=_RES_DT)
        coefs = np.zeros(max(1, batch.n_coefs), dtype=np.float64)
        b = batch.struct()
        check(self.ctx.lib.rrg_eval(self.h, C.byref(b), precision, res.ctypes.data_as(C.POINTER(Result)),
                                    coefs.ctypes.data_as(C.POINTER(C.c_double))), "rrg_eval")
        return decode_results(res, coefs, batch)

    def submit(self, batch: EncodedBatch, precision: int, res: np.ndarray, coefs: np.ndarray):
        """Asynchronous round; complete it with wait().  Buffers must stay alive."""
        b = batch.struct()
        check(self.ctx.lib.rrg_round_submit(self.h, C.byref(b), precision, res.ctypes.data_as(C.POINTER(Result)),
                                            coefs.ctypes.data_as(C.POINTER(C.c_double))), "rrg_round_submit")

    def wait(self, timeout_ms: int = -1):
        check(self.ctx.lib.rrg_round_wait(self.ctx.h, timeout_ms), "rrg_round_wait")

    def predict(self, tree: str) -> np.ndarray:
        batch = encode([tree], tuned=False)
        out = np.zeros(self.n, dtype=np.float64)
        b = batch.struct()
        check(self.ctx.lib.rrg_predict(self.h, C.byref(b), out.ctypes.data_as(C.POINTER(C.c_double))), "rrg_predict")
        return out

    def close(self):
        if self.h:
            self.ctx.lib.rrg_dataset_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def result_dtype() -> np.dtype:
    return _RES_DT


# ------------------------------------------------------ launch-shape tuner --
EVAL_WAVES = _lib.RRG_KNOB_EVAL_WAVES
FAC_GROUP = _lib.RRG_KNOB_FAC_GROUP
PAIR_UNIT = _lib.RRG_KNOB_PAIR_UNIT
FAC_STAGE = _lib.RRG_KNOB_FAC_STAGE


def tune_mode(on: bool) -> None:
    """Time every result-invariant launch shape on first use (on, the default)
    or keep the built-in shapes (off)."""
    lib = _lib.load()
    check(lib.rrg_tune_set_mode(_lib.RRG_TUNE_ON if on else _lib.RRG_TUNE_OFF), "rrg_tune_set_mode")


def tune_pin(knob: int, bucket: int, value: int) -> None:
    """Fix a knob's value in a bucket (0 releases it)."""
    lib = _lib.load()
    check(lib.rrg_tune_pin(knob, bucket, value), "rrg_tune_pin")


def tune_reset() -> None:
    lib = _lib.load()
    check(lib.rrg_tune_reset(), "rrg_tune_reset")


def tune_report() -> list[dict]:
    """The tuner's choices: knob, bucket, row class, value and the timed shapes (ms)."""
    lib = _lib.load()
    need = lib.rrg_tune_report(None, 0)
    buf = C.create_string_buffer(int(need))
    lib.rrg_tune_report(buf, need)
    out = []
    for line in buf.value.decode().splitlines():
        parts = line.split()
        e = {"knob": parts[0]}
        for kv in parts[1:]:
            k, v = kv.split("=", 1)
            if k == "ms":
                e["ms"] = {int(a): float(b) for a, b in (t.split(":") for t in v.split(","))}
            else:
                e[k] = int(v)
        out.append(e)
    return out

