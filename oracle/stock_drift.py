"""ORACLE measurement (test infrastructure only): how far the reference's
results move when it is built with stock arithmetic (the C library's
transcendentals, index-order sums; `oracle/build_ref.sh --stock`) instead of
the pinned arithmetic the golden fixtures were made with.

For every case of tests/golden/fitness.json it scores the tree with the
stock build's tune_constants + fitness and counts the fitness triples that
differ from the golden ones by more than `rel` relative; for every full fit
of tests/golden/fit.json it reruns the reference's fit and compares the
model string and fit-call count.  Needs oracle/_ref/librr_ref_stock.so
(built only where the reference checkout exists).

    python oracle/stock_drift.py
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
GOLDEN = HERE.parent / "tests" / "golden"
LIB = HERE / "_ref" / "librr_ref_stock.so"


def fv(f):
    return (1 + f[0]) * (1 + f[1]) * (1 + f[2] * 1e-3)


def measure(rel: float = 1e-10) -> dict:
    lib = C.CDLL(str(LIB))
    dp = C.POINTER(C.c_double)
    buf = C.create_string_buffer(1 << 24)
    out3 = (C.c_double * 3)()
    sets = json.loads((GOLDEN / "fitness.json").read_text())
    report = {"rel": rel, "fitness": {}, "fits": {}}
    for name, spec in sets.items():
        X = np.array(spec["X"], dtype=np.float64)
        y = np.ascontiguousarray(np.array(spec["y"], dtype=np.float64))
        Xc = np.ascontiguousarray(X.T)
        n, d = X.shape
        row = {"cases": 0, "differ": 0, "max_rel": 0.0, "sentinel_changed": 0, "size_changed": 0}
        for case in spec["cases"]:
            for tuned, key in ((1, "tuned"), (0, "untuned")):
                r = lib.ref_tune_fitness(Xc.ctypes.data_as(dp), y.ctypes.data_as(dp), n, d, case["tree"].encode(),
                                         tuned, int(spec["classification"]), out3, buf, len(buf))
                if r < 0:
                    raise RuntimeError(buf.value[:300])
                got = [out3[0], out3[1], int(out3[2])]
                want = case[key]["fit"]
                row["cases"] += 1
                if (got[0] == 1000) != (want[0] == 1000):
                    row["sentinel_changed"] += 1
                    row["differ"] += 1
                    continue
                if got[2] != want[2]:
                    row["size_changed"] += 1
                a, b = fv(got), fv(want)
                e = abs(a - b) / abs(b) if b else abs(a - b)
                if not np.isfinite(e):
                    e = 0.0 if a == b else float("inf")
                row["max_rel"] = max(row["max_rel"], e)
                if e > rel or got[2] != want[2]:
                    row["differ"] += 1
        report["fitness"][name] = row
    fits = json.loads((GOLDEN / "fit.json").read_text())
    data = fits["toy_data"]
    for name, spec in fits.items():
        if name == "toy_data":
            continue
        cfg = spec["cfg"]
        if "X" in spec:
            X, y = np.array(spec["X"]), np.array(spec["y"])
        else:
            X, y = np.array(data["Xtr"]), np.array(data["ytr"])
        X = np.ascontiguousarray(X, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        n, d = X.shape
        pred = np.zeros(n)
        calls = lib.ref_fit(X.ctypes.data_as(dp), y.ctypes.data_as(dp), n, d, cfg["cls"], cfg["max_fit_calls"],
                            1 << 30, C.c_double(cfg["cp"]), cfg["max_complexity"], C.c_double(cfg["sample_size"]),
                            cfg["seed"], buf, len(buf), pred.ctypes.data_as(dp))
        model = buf.value.decode().split("\n")[0]
        report["fits"][name] = {"model_same": model == spec["model"], "fit_calls_same": calls == spec["fit_calls"],
                                "model": model, "golden_model": spec["model"]}
    return report


if __name__ == "__main__":
    if not LIB.exists():
        sys.exit(f"{LIB} is missing: run oracle/build_ref.sh --stock where the reference checkout exists")
    print(json.dumps(measure(), indent=1))
