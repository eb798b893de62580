"""The rule by which the FP64 path skips the column-pivoted QR
(sentinel_classify_kernel, csrc/device/plain.cu): when column 0's norm is
NaN or any column's norm is +inf, and every column has a non-trivial tail,
the oracle's QR (oracle/colpiv_qr.h) returns all-NaN coefficients at full
rank.  Checked here on the oracle with the column statistics restated in
numpy, over the golden fitness sets and a random-tree batch (CPU only)."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle
from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import encode


def decided(cols, rows):
    if not cols or rows < len(cols) + 3:
        return False
    tails, inf_norm, nan0 = True, False, False
    for j, c in enumerate(cols):
        a = np.abs(c)
        tails &= bool(((a[1:] > 1e-150) | ~np.isfinite(c[1:])).any())
        if np.isnan(c).any():
            nan0 |= j == 0
        elif (~(a <= 1.35e154)).any():
            inf_norm = True
    return tails and (nan0 or inf_norm)


def check(lib, X, y, trees):
    out = pyoracle.OracleDataset(X, y).evaluate(encode(trees, tuned=True), threads=4)
    buf = C.create_string_buffer(1 << 20)
    n_dec = 0
    with np.errstate(all="ignore"):
        for i, tr in enumerate(trees):
            assert lib.rrh_rewrite(tr.encode(), 5, buf, len(buf)) >= 0
            facs = [f.split("\t")[-1] for f in buf.value.decode().split("\n") if f]
            cols = [np.broadcast_to(synth.eval_tree(f, X), (X.shape[0],)).astype(float) for f in facs]
            if decided(cols, X.shape[0]):
                n_dec += 1
                co = out["coefs"][i]
                assert np.isnan(co).all() and out["rank"][i] == len(co) and out["loss"][i] == 1000, tr
    return n_dec


@pytest.mark.parametrize("name", ["toy", "rand257x3", "cls120x4"])
def test_rule_on_golden_sets(lib, golden, name):
    spec = golden("fitness")[name]
    assert check(lib, np.array(spec["X"]), np.array(spec["y"]), [c["tree"] for c in spec["cases"]]) > 0


def test_rule_on_random_trees(lib):
    X, y, trees, _ = synth.batched_fitness(n=3000, d=5, n_trees=600, seed=9, max_size=50)
    assert check(lib, X, y, trees) > 100
