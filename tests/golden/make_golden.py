"""Generates the golden fixtures of tests/golden/ from the reference itself.

Runs only where the reference checkout exists (see oracle/build_ref.sh): it
builds oracle/_ref/librr_ref.so with oracle/build_ref.sh (the reference's own
rils_rols_cpp.cpp and node.cpp, unmodified, against the self-written Eigen
subset in oracle/eigen_shim/) and records, for seeded inputs:
  * fit.json        full fits (model string, fit calls, predictions)
  * fitness.json    tune_constants + fitness per candidate tree
  * candidates.json all_candidates lists (sha256 of the text + count + head)
  * rewrite.json    expand / simplify / normalize / clean-up / factor split
Usage: python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "rils-rols_gb300"))
from rils_rols_gb300 import synth  # noqa: E402

# the reference checkout: first argument, else what oracle/build_ref.sh finds
# (environment variable RILS_ROLS_REFERENCE or the recipe's default)
subprocess.run([str(REPO / "oracle" / "build_ref.sh")] + sys.argv[1:2], check=True)
lib = C.CDLL(str(REPO / "oracle" / "_ref" / "librr_ref.so"))
dp = C.POINTER(C.c_double)
BUF = C.create_string_buffer(1 << 26)


def call(fn, *args):
    r = fn(*args, BUF, len(BUF))
    if r < 0:
        raise RuntimeError(BUF.value[:300])
    return BUF.value.decode()


def ref_fit(X, y, cls, max_fit_calls, cp, max_complexity, sample_size, seed):
    X = np.ascontiguousarray(X, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    n, d = X.shape
    pred = np.zeros(n)
    fc = lib.ref_fit(X.ctypes.data_as(dp), y.ctypes.data_as(dp), n, d, int(cls), max_fit_calls, 1 << 30,
                     C.c_double(cp), max_complexity, C.c_double(sample_size), seed, BUF, len(BUF),
                     pred.ctypes.data_as(dp))
    model, prefix = BUF.value.decode().split("\n")
    return {"model": model, "prefix": prefix, "fit_calls": fc, "pred": pred.tolist()}


def tree_suite(rng, count, d, cls=False, max_size=30):
    ops2 = synth.BINARY + (synth.CLS_BINARY if cls else ())
    out = []
    for _ in range(count):
        s = int(rng.integers(1, max_size + 1))
        out.append(synth.random_tree(rng, s, d, unary=synth.UNARY + ("sqr",), binary=ops2, p_var=0.6))
    return out


SPECIAL = [  # rank-deficient, constant, non-finite and degenerate candidates
    "add x0 x0", "add mul sin x0 sin x0 mul cos x0 cos x0", "div x0 x0", "sub x1 x1", "c:3.5", "x0",
    "add x0 mul c:2 x0", "ln sub x0 c:1000", "div c:1 sub x0 x0", "sqrt mul c:-1 sqr x1",
    "add add x0 x1 add x0 x1", "mul add x0 c:1 x1", "mul x1 add x0 c:1", "mul add x0 x1 sub x0 x1",
    "exp mul c:100 x0", "add exp mul c:800 x1 x0", "add x0 sub c:0 x0", "mul c:0 x0", "add c:1e-13 x0",
]


def main():
    fits = {}
    Xtr, Xte, ytr, yte = synth.toy_example()
    fits["toy_100000"] = {"cfg": dict(cls=0, max_fit_calls=100000, cp=0.001, max_complexity=50, sample_size=1.0,
                                      seed=12345), **ref_fit(Xtr, ytr, 0, 100000, 0.001, 50, 1.0, 12345)}
    for seed in (0, 1, 7):
        fits[f"toy_3000_s{seed}"] = {"cfg": dict(cls=0, max_fit_calls=3000, cp=0.001, max_complexity=50,
                                                 sample_size=1.0, seed=seed),
                                     **ref_fit(Xtr, ytr, 0, 3000, 0.001, 50, 1.0, seed)}
    fits["toy_sample_half"] = {"cfg": dict(cls=0, max_fit_calls=4000, cp=0.001, max_complexity=50, sample_size=0.5,
                                           seed=3), **ref_fit(Xtr, ytr, 0, 4000, 0.001, 50, 0.5, 3)}
    Xc, yc, _ = synth.classifier(n=200, d=6, seed=11)
    fits["cls_200x6"] = {"cfg": dict(cls=1, max_fit_calls=3000, cp=0.001, max_complexity=20, sample_size=1.0,
                                     seed=5), "X": Xc.tolist(), "y": yc.tolist(),
                         **ref_fit(Xc, yc, 1, 3000, 0.001, 20, 1.0, 5)}
    fits["toy_data"] = {"Xtr": Xtr.tolist(), "ytr": ytr.tolist(), "Xte": Xte.tolist(), "yte": yte.tolist()}
    (HERE / "fit.json").write_text(json.dumps(fits))

    # per-candidate fitness
    rng = np.random.default_rng(2024)
    sets = {}
    datasets = {
        "toy": (Xtr, ytr, False),
        "rand257x3": None,
        "cls120x4": None,
        "tiny3x2": None,
    }
    Xr = np.random.default_rng(7).standard_normal((257, 3))
    yr = np.sin(Xr[:, 0]) * 2 + Xr[:, 1] * Xr[:, 2] + 0.1 * np.random.default_rng(8).standard_normal(257)
    datasets["rand257x3"] = (Xr, yr, False)
    Xk, yk, _ = synth.classifier(n=120, d=4, seed=3)
    datasets["cls120x4"] = (Xk, yk, True)
    Xt = np.array([[1.0, 2.0], [3.0, -1.0], [0.5, 4.0]])
    datasets["tiny3x2"] = (Xt, np.array([1.0, 2.0, 0.0]), False)
    out3 = (C.c_double * 3)()
    for name, (X, y, cls) in datasets.items():
        d = X.shape[1]
        trees = tree_suite(rng, 150, d, cls) + [t for t in SPECIAL if max(
            [int(tok[1:]) for tok in t.split() if tok[0] == "x"] + [-1]) < d]
        Xcol = np.ascontiguousarray(X.T)
        yy = np.ascontiguousarray(y)
        rows = []
        for t in trees:
            rec = {"tree": t}
            for tuned in (1, 0):
                r = lib.ref_tune_fitness(Xcol.ctypes.data_as(dp), yy.ctypes.data_as(dp), X.shape[0], d, t.encode(),
                                         tuned, int(cls), out3, BUF, len(BUF))
                if r < 0:
                    raise RuntimeError(BUF.value[:300])
                s, p = BUF.value.decode().split("\n")
                rec["tuned" if tuned else "untuned"] = {"fit": [out3[0], out3[1], int(out3[2])], "model": s,
                                                        "prefix": p}
            rows.append(rec)
        sets[name] = {"X": X.tolist(), "y": y.tolist(), "classification": cls, "cases": rows}
    (HERE / "fitness.json").write_text(json.dumps(sets))

    # candidate lists
    crng = np.random.default_rng(99)
    cands = []
    for i in range(40):
        cls = i % 4 == 3
        t = synth.random_tree(crng, int(crng.integers(1, 14)), 3,
                              binary=synth.BINARY + (synth.CLS_BINARY if cls else ()), p_var=0.6)
        for ls in (0, 1):
            txt = call(lib.ref_candidates, t.encode(), ls, 3, int(cls))
            lines = txt.split("\n")
            cands.append({"tree": t, "local_search": ls, "d": 3, "classification": int(cls),
                          "sha256": hashlib.sha256(txt.encode()).hexdigest(), "count": len(lines) - 1,
                          "head": lines[:5]})
    (HERE / "candidates.json").write_text(json.dumps(cands))

    # rewriting primitives
    wrng = np.random.default_rng(5)
    rew = []
    for i in range(250):
        cls = i % 5 == 4
        t = synth.random_tree(wrng, int(wrng.integers(1, 26)), 3, unary=synth.UNARY + ("sqr",),
                              binary=synth.BINARY + (synth.CLS_BINARY if cls else ()), p_var=0.5)
        rew.append({"tree": t, "out": [call(lib.ref_rewrite, t.encode(), w) for w in range(6)]})
    (HERE / "rewrite.json").write_text(json.dumps(rew))
    for f in ("fit.json", "fitness.json", "candidates.json", "rewrite.json"):
        print(f, (HERE / f).stat().st_size)


if __name__ == "__main__":
    main()
