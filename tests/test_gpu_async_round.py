"""Mixed and certified rounds whose second half the device decides
(rrg_context_set_async on, the default: residual-pass list, FP64 re-scoring
list, table columns to evaluate and QR buckets compacted on the device)
against the same rounds decided on the host (off: two read-backs per round):
every result field and coefficient the same bits, and the same round
statistics."""
import gzip

import numpy as np
import pytest

from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import CERTIFIED, MIXED, Context, encode

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def same(a, b, tag):
    for f in ("loss", "rmse", "size", "rank", "flags"):
        assert np.array_equal(a[f], b[f], equal_nan=True), (tag, f)
    for i, (x, y) in enumerate(zip(a["coefs"], b["coefs"])):
        assert np.array_equal(x, y, equal_nan=True), (tag, "coefs", i)


def compare(ctx, ds, trees, tag):
    b = encode(trees, tuned=True)
    for prec in (CERTIFIED, MIXED):
        ctx.set_async(False)
        want = ds.evaluate(b, prec)
        st_want = ctx.last_round_stats()
        ctx.set_async(True)
        got = ds.evaluate(b, prec)
        st_got = ctx.last_round_stats()
        same(got, want, (tag, prec))
        for k in ("fp64_rescored", "residual_pass", "plain_routed", "rescore_reasons"):
            assert st_got[k] == st_want[k], (tag, prec, k, st_got[k], st_want[k])
        # a second device-decided round on the same context: no stale state
        again = ds.evaluate(b, prec)
        same(again, want, (tag, prec, "again"))
    return st_got


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    c.set_mixed_min_rows(0)
    c.set_column_cache(False)  # both forms evaluate the whole table every time
    yield c
    c.close()


def test_async_matches_host_decided_1m_round(ctx):
    X, y = synth.regression_1m()
    rounds = {}
    for line in gzip.open(GOLDEN / "ls_rounds_regression_1m.txt.gz", "rt").read().splitlines():
        r, t = line.split("\t")
        rounds.setdefault(int(r), []).append(t)
    ds = ctx.dataset(X, y)
    st = compare(ctx, ds, rounds[4] + rounds[5], "1M rounds 4-5")
    assert st["fp64_rescored"] > 0  # the re-scoring lane ran
    ds.close()


def test_async_matches_host_decided_random_trees(ctx):
    # many NaN producers and sentinel shortcuts
    X, y, trees, _ = synth.batched_fitness(n=100_000, d=10, n_trees=2048, seed=77)
    ds = ctx.dataset(X, y)
    st = compare(ctx, ds, trees, "random trees 100k")
    assert st["fp64_rescored"] > 0
    ds.close()


def test_async_matches_host_decided_small(ctx):
    rng = np.random.default_rng(3)
    n = 12_000
    X = rng.uniform(-3, 3, (n, 4))
    y = X[:, 0] * np.exp(0.3 * X[:, 1]) - np.cos(X[:, 2]) + 0.01 * rng.standard_normal(n)
    trees = [synth.random_tree(rng, int(rng.integers(3, 30)), 4) for _ in range(600)]
    trees += ["add x0 x0", "add x1 mul c:2 x1", "ln sub x0 c:100", "add sqrt x0 x1"]
    ds = ctx.dataset(X, y)
    compare(ctx, ds, trees, "small")
    ds.close()
