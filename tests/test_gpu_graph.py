"""Rounds run as CUDA graphs (rrg_context_set_graph) against the same rounds
launched directly: the same bits in every result field and coefficient, for
small FP64 rounds (the classifier's shape), for certified mixed rounds
whose second half the device decides, and for a certified round of fewer
than 64 candidates (host-decided without graphs, device-decided as a
graph); the statistics report that the round
really ran as a graph, and a second round on the same context (the previous
graph updated or rebuilt) gives the same results again."""
import numpy as np
import pytest

from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import CERTIFIED, PLAIN, Context, encode

pytestmark = pytest.mark.gpu


def same(a, b, tag):
    for f in ("loss", "rmse", "size", "rank", "flags"):
        assert np.array_equal(a[f], b[f], equal_nan=True), (tag, f)
    for i, (x, y) in enumerate(zip(a["coefs"], b["coefs"])):
        assert np.array_equal(x, y, equal_nan=True), (tag, "coefs", i)


def run(X, y, trees, prec, tag, min_rows=None):
    ctx = Context(0)
    try:
        ctx.set_column_cache(False)  # the captured rounds evaluate the whole table (the cache's own test covers both)
        if min_rows is not None:
            ctx.set_mixed_min_rows(min_rows)
        ds = ctx.dataset(X, y)
        b = encode(trees, tuned=True)
        want = ds.evaluate(b, prec)  # direct launches (also settles launch-shape trials)
        ctx.set_graph(True)
        for i in range(3):
            got = ds.evaluate(b, prec)
            assert ctx.last_round_stats()["graph"], (tag, i)
            same(got, want, (tag, i))
        # another batch on the same context: the graph changes shape
        b2 = encode(trees[: len(trees) // 2], tuned=True)
        got2 = ds.evaluate(b2, prec)
        ctx.set_graph(False)
        want2 = ds.evaluate(b2, prec)
        same(got2, want2, (tag, "half"))
        ds.close()
    finally:
        ctx.close()


def test_graph_small_fp64_rounds():
    X, lab, _ = synth.classifier(n=569, d=30, seed=12345)
    rng = np.random.default_rng(8)
    trees = [synth.random_tree(rng, int(rng.integers(3, 20)), 30, binary=synth.BINARY + synth.CLS_BINARY)
             for _ in range(400)]
    run(X, lab, trees, PLAIN, "classifier shape")


def test_graph_certified_mixed_round():
    X, y, trees, _ = synth.batched_fitness(n=60_000, d=6, n_trees=1500, seed=31)
    run(X, y, trees, CERTIFIED, "certified mixed", min_rows=0)


def test_graph_small_certified_round():
    # fewer than 64 candidates: without graphs the round reads its flags back
    # (host-decided second half); as a graph it decides them on the device
    X, y, trees, _ = synth.batched_fitness(n=60_000, d=6, n_trees=48, seed=37)
    b = encode(trees, tuned=True)
    direct = Context(0)
    graph = Context(0)
    try:
        for c in (direct, graph):
            c.set_mixed_min_rows(0)
            c.set_column_cache(False)
        want = direct.dataset(X, y).evaluate(b, CERTIFIED)
        graph.set_graph(True)
        ds = graph.dataset(X, y)
        same(ds.evaluate(b, CERTIFIED), want, "first graph round (may allocate, then run directly)")
        for i in range(3):
            got = ds.evaluate(b, CERTIFIED)
            assert graph.last_round_stats()["graph"], i
            same(got, want, ("small certified", i))
    finally:
        direct.close()
        graph.close()
