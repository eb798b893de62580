"""The rules by which the FP64 path skips the column-pivoted QR
(sentinel_classify_kernel and nan_gram_decide_kernel, csrc/device/plain.cu):
with every column's tail non-trivial, (A) a NaN norm in column 0 or an
infinite norm anywhere, or (B) a NaN column further right with well
conditioned finite columns, make the oracle's QR (oracle/colpiv_qr.h)
return all-NaN coefficients at full rank.  Checked on the oracle with the
column statistics restated in numpy, over the golden fitness sets, a
random-tree batch and the local-search candidates (CPU only)."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle
from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import encode


def well_conditioned(cols):
    """The Gram certificate of nan_gram_decide_kernel: pivoted Cholesky of the
    FP64 Gram matrix, every pivot above 1e-8 of its column's squared norm and
    1e-24 of the largest."""
    G = np.array([[float(np.dot(a, b)) for b in cols] for a in cols])
    d0 = np.diag(G).copy()
    maxd = d0.max()
    if not (0 < maxd < 1e300):
        return False
    piv = list(range(len(cols)))
    for s in range(len(cols)):
        q = s + int(np.argmax(np.diag(G)[s:]))
        dp = G[q, q]
        if not (dp > 1e-8 * d0[piv[q]]) or not (dp > 1e-24 * maxd):
            return False
        G[[s, q]] = G[[q, s]]
        G[:, [s, q]] = G[:, [q, s]]
        piv[s], piv[q] = piv[q], piv[s]
        G[s + 1:, s] /= np.sqrt(dp)
        G[s + 1:, s + 1:] -= np.outer(G[s + 1:, s], G[s + 1:, s])
    return True


def decided(cols, rows):
    """(rule, decided): rule "A" for a NaN column 0 or an infinite norm, "B"
    for a NaN column further right with well-conditioned finite columns."""
    if not cols or rows < len(cols) + 3:
        return None
    tails, inf_norm, nan0, nan_any = True, False, False, False
    for j, c in enumerate(cols):
        a = np.abs(c)
        tails &= bool(((a[1:] > 1e-150) | ~np.isfinite(c[1:])).any())
        if np.isnan(c).any():
            nan0 |= j == 0
            nan_any = True
        elif (~(a <= 1.35e154)).any():
            inf_norm = True
    if not tails:
        return None
    if nan0 or inf_norm:
        return "A"
    finite = [c for c in cols if not np.isnan(c).any()]
    if nan_any and len(finite) + 1 <= 9 and well_conditioned(finite + [np.ones(rows)]):
        return "B"
    return None


def check(lib, X, y, trees):
    out = pyoracle.OracleDataset(X, y).evaluate(encode(trees, tuned=True), threads=4)
    buf = C.create_string_buffer(1 << 20)
    n_dec = {"A": 0, "B": 0}
    with np.errstate(all="ignore"):
        for i, tr in enumerate(trees):
            assert lib.rrh_rewrite(tr.encode(), 5, buf, len(buf)) >= 0
            facs = [f.split("\t")[-1] for f in buf.value.decode().split("\n") if f]
            cols = [np.broadcast_to(synth.eval_tree(f, X), (X.shape[0],)).astype(float) for f in facs]
            rule = decided(cols, X.shape[0])
            if rule:
                n_dec[rule] += 1
                co = out["coefs"][i]
                assert np.isnan(co).all() and out["rank"][i] == len(co) and out["loss"][i] == 1000, (rule, tr)
    return n_dec


@pytest.mark.parametrize("name", ["toy", "rand257x3", "cls120x4"])
def test_rule_on_golden_sets(lib, golden, name):
    spec = golden("fitness")[name]
    assert check(lib, np.array(spec["X"]), np.array(spec["y"]), [c["tree"] for c in spec["cases"]])["A"] > 0


def test_rule_on_random_trees(lib):
    X, y, trees, _ = synth.batched_fitness(n=3000, d=5, n_trees=600, seed=9, max_size=50)
    n_dec = check(lib, X, y, trees)
    assert n_dec["A"] > 100 and n_dec["B"] > 0


def test_rule_on_local_search_candidates(lib):
    X, y = synth.regression_1m(n=20000)
    n_dec = check(lib, X, y, synth.ls_round_batch(d=5))
    assert n_dec["A"] > 0 and n_dec["B"] > 0
