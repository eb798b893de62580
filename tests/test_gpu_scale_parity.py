"""Device results at the benchmark's own shapes against the oracle.

The oracle side flattens the trees with its own encoder
(oracle/tree_encode.py) and scores them with oracle/rrg_oracle.c on every
host thread; the device side scores whole rounds through the C ABI, exactly
as the benchmark does, and a seeded sample of the candidates is compared:

* batched fitness, n = 100k, d = 10: the 8192 random trees (sizes 3..50 over
  + - * / sin cos ln exp sqrt) in one round, 512 of them checked;
* the 1M-row regression search: its eight local-search rounds, one call per
  round, 96 candidates checked.

Plain FP64 must be bit-identical to the oracle in every round, whatever its
size (round 0 of the 1M-row search has 264 candidates, the batched round
8192; every QR runs in the same QSUM order).  The certified mixed form must
be within 1e-6 relative in the penalised fitness with the same NaN
sentinels, and the sample's best candidate the same.
"""
import gzip
import os

import numpy as np
import pytest

from oracle import pyoracle, tree_encode
from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import CERTIFIED, PLAIN, Context, encode

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

REL_CERT = 1e-6
THREADS = os.cpu_count() or 1


def fval(r):
    return (1 + r["loss"]) * (1 + r["rmse"]) * (1 + r["size"] * 1e-3)


def pick(out, idx):
    return {k: np.asarray(v)[idx] for k, v in out.items() if k != "coefs"}


def check(dev_plain, dev_cert, ora, tag):
    # plain FP64: bit for bit
    for f in ("size", "rank"):
        assert np.array_equal(dev_plain[f], ora[f]), (tag, f)
    for f in ("loss", "rmse"):
        a, b = dev_plain[f], ora[f]
        exact = (a == b) | ((a != a) & (b != b))
        assert np.all(exact), (tag, f, np.flatnonzero(~exact)[:5])
    assert np.array_equal(dev_plain["loss"] == 1000, ora["loss"] == 1000), tag
    # certified: same sentinels, fitness within 1e-6
    sent = ora["loss"] == 1000
    assert np.array_equal(dev_cert["loss"] == 1000, sent), tag
    ok = ~sent & np.isfinite(fval(ora))
    err = np.abs(fval(dev_cert)[ok] - fval(ora)[ok]) / fval(ora)[ok]
    assert np.all(err <= REL_CERT), (tag, float(err.max()))
    best = lambda r: int(np.argmin(np.where(ok, fval(r), np.inf)))  # noqa: E731
    assert best(dev_cert) == best(ora) == best(dev_plain), tag


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def test_batched_fitness_100k_d10(ctx):
    X, y, trees, _ = synth.batched_fitness(n=100_000, d=10, n_trees=8192, seed=12345)
    ds = ctx.dataset(X, y)
    b = encode(trees, tuned=True)
    plain, cert = ds.evaluate(b, PLAIN), ds.evaluate(b, CERTIFIED)
    idx = np.sort(np.random.default_rng(21).choice(len(trees), 512, replace=False))
    ora = pyoracle.OracleDataset(X, y).evaluate(tree_encode.encode([trees[i] for i in idx]), threads=THREADS)
    check(pick(plain, idx), pick(cert, idx), ora, "8192 random trees, n=100k, d=10")
    ds.close()


def test_regression_1m_rounds(ctx):
    X, y = synth.regression_1m()
    rounds = {}
    for line in gzip.open(GOLDEN / "ls_rounds_regression_1m.txt.gz", "rt").read().splitlines():
        r, t = line.split("\t")
        rounds.setdefault(int(r), []).append(t)
    ds = ctx.dataset(X, y)
    plain, cert, trees = [], [], []
    for r in sorted(rounds):
        b = encode(rounds[r], tuned=True)
        plain.append(ds.evaluate(b, PLAIN))
        cert.append(ds.evaluate(b, CERTIFIED))
        trees += rounds[r]
    cat = lambda outs: {k: np.concatenate([o[k] for o in outs]) for k in ("loss", "rmse", "size", "rank")}  # noqa
    plain, cert = cat(plain), cat(cert)
    idx = np.sort(np.random.default_rng(22).choice(len(trees), 96, replace=False))
    ora = pyoracle.OracleDataset(X, y).evaluate(tree_encode.encode([trees[i] for i in idx]), threads=THREADS)
    check(pick(plain, idx), pick(cert, idx), ora, "1M-row local-search rounds")
    ds.close()
