"""Factor columns kept across rounds (rrg_context_set_column_cache): the
rounds of a search trajectory read the columns earlier rounds evaluated (the
double-float table, the FP64 table and the FP64 re-scoring lane of mixed
rounds), and every result is the same bits as with the cache off, for each precision,
under eviction pressure (a table limit of a few columns), across a switch of
datasets, as CUDA graphs, and against the oracle."""
import numpy as np
import pytest

from oracle import pyoracle
from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import CERTIFIED, MIXED, PLAIN, Context, candidates, encode

pytestmark = pytest.mark.gpu

N = 20000


def trajectory_batches(limit=None):
    out = []
    for t in synth.REGRESSION_1M_TRAJECTORY:
        cs = candidates(t, 5, local_search=True)
        out.append(encode(cs[:limit] if limit else cs, tuned=True))
    return out


@pytest.fixture(scope="module")
def data():
    X, y = synth.regression_1m(n=N)
    return X, y, trajectory_batches(400)


def run(ctx, X, y, batches, prec):
    ds = ctx.dataset(X, y)
    res, stats = [], []
    for b in batches:
        res.append(ds.evaluate(b, prec))
        stats.append(ctx.last_round_stats())
    ds.close()
    return res, stats


def same(a, b):
    for key in ("loss", "rmse"):
        x, z = a[key], b[key]
        if not np.all((x == z) | (np.isnan(x) & np.isnan(z))):
            return False
    if not (np.array_equal(a["size"], b["size"]) and np.array_equal(a["rank"], b["rank"])):
        return False
    for p, q in zip(a["coefs"], b["coefs"]):
        if not np.all((p == q) | (np.isnan(p) & np.isnan(q))):
            return False
    return True


@pytest.mark.parametrize("prec", [PLAIN, CERTIFIED, MIXED])
def test_cached_rounds_are_bit_identical(data, prec):
    X, y, batches = data
    on = Context(0)
    on.set_mixed_min_rows(0)
    off = Context(0)
    off.set_mixed_min_rows(0)
    off.set_column_cache(False)
    r_on, s_on = run(on, X, y, batches, prec)
    r_off, s_off = run(off, X, y, batches, prec)
    for i, (a, b) in enumerate(zip(r_on, r_off)):
        assert same(a, b), f"round {i}"
    key = "cache64_hits" if prec == PLAIN else "cache_hits"
    assert s_on[0][key] == 0
    assert sum(s[key] for s in s_on[1:]) > 0  # later rounds read kept columns
    assert all(s[key] == 0 for s in s_off)
    if prec != PLAIN:
        # cross-pair sums of earlier rounds read again
        assert sum(s["pair_hits"] for s in s_on[1:]) > 0 and all(s["pair_hits"] == 0 for s in s_off)
        # the FP64 re-scoring lane: columns it evaluated in one round are
        # stored when the next starts, and later lanes copy them in
        assert sum(s["fp64_rescored"] for s in s_on) > 0
        assert sum(s["cache64_hits"] for s in s_on[2:]) > 0
        assert all(s["cache64_hits"] == 0 for s in s_off)
    on.close()
    off.close()


def test_eviction_pressure_and_dataset_switch(data):
    X, y, batches = data
    ref = Context(0)
    ref.set_mixed_min_rows(0)
    ref.set_column_cache(False)
    r_ref, _ = run(ref, X, y, batches[:4], CERTIFIED)
    p_ref, _ = run(ref, X, y, batches[:4], PLAIN)
    ref.close()
    # a table of a few columns: sub-rounds without shared columns, slots
    # replaced in every round; the same bits as the whole-round table
    tight = Context(0)
    tight.set_mixed_min_rows(0)
    tight.set_limits(1 << 20, 1 << 20)
    r_t, s_t = run(tight, X, y, batches[:4], CERTIFIED)
    assert sum(s["cache_hits"] for s in s_t[1:]) > 0
    for a, b in zip(r_t, r_ref):
        assert same(a, b)
    p_t, _ = run(tight, X, y, batches[:4], PLAIN)
    for a, b in zip(p_t, p_ref):
        assert same(a, b)
    tight.close()
    # two datasets in turn on one context: each round sees its own columns
    rng = np.random.default_rng(3)
    X2 = rng.uniform(-3, 3, X.shape)
    y2 = X2[:, 0] - np.cos(X2[:, 1]) + 0.01 * rng.standard_normal(N)
    alt = Context(0)
    alt.set_mixed_min_rows(0)
    d1, d2 = alt.dataset(X, y), alt.dataset(X2, y2)
    fresh = Context(0)
    fresh.set_mixed_min_rows(0)
    fresh.set_column_cache(False)
    f2 = fresh.dataset(X2, y2)
    for i, b in enumerate(batches[:4]):
        assert same(d1.evaluate(b, CERTIFIED), r_ref[i])
        assert same(d2.evaluate(b, CERTIFIED), f2.evaluate(b, CERTIFIED))
    d1.close()
    d2.close()
    f2.close()
    alt.close()
    fresh.close()


def test_graph_rounds_with_cache(data):
    X, y, batches = data
    g = Context(0)
    g.set_mixed_min_rows(0)
    g.set_graph(True)
    plain = Context(0)
    plain.set_mixed_min_rows(0)
    plain.set_column_cache(False)
    r_g, s_g = run(g, X, y, batches, CERTIFIED)
    r_p, _ = run(plain, X, y, batches, CERTIFIED)
    for a, b in zip(r_g, r_p):
        assert same(a, b)
    assert any(s["graph"] for s in s_g)
    g.close()
    plain.close()


def test_cached_round_matches_oracle(data):
    X, y, _ = data
    b_all = trajectory_batches(120)
    ctx = Context(0)
    ds = ctx.dataset(X, y)
    for b in b_all[:5]:
        ds.evaluate(b, PLAIN)
    assert ctx.last_round_stats()["cache64_hits"] > 0
    last = b_all[5]
    dev = ds.evaluate(last, PLAIN)
    assert ctx.last_round_stats()["cache64_hits"] > 0
    ora = pyoracle.OracleDataset(X, y).evaluate(last, threads=8)
    for key in ("loss", "rmse"):
        assert np.all((dev[key] == ora[key]) | (np.isnan(dev[key]) & np.isnan(ora[key]))), key
    assert np.array_equal(dev["size"], ora["size"])
    ds.close()
    ctx.close()


def test_clear_and_switch_off(data):
    X, y, batches = data
    ctx = Context(0)
    ctx.set_mixed_min_rows(0)
    ds = ctx.dataset(X, y)
    a = ds.evaluate(batches[1], CERTIFIED)
    b = ds.evaluate(batches[1], CERTIFIED)  # every column kept
    assert ctx.last_round_stats()["cache_evals"] == 0
    ctx.clear_column_cache()
    c = ds.evaluate(batches[1], CERTIFIED)
    assert ctx.last_round_stats()["cache_hits"] == 0
    assert same(a, b) and same(a, c)
    ds.close()
    ctx.close()
