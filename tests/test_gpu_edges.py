"""Edge cases of the device path against the oracle: an empty batch, datasets
of one to three rows, a constant target (SST = 0), untuned candidates in the
mixed forms, and a candidate with more than 15 factors (the widest QR
bucket)."""
import numpy as np
import pytest

from oracle import pyoracle
from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import CERTIFIED, MIXED, PLAIN, Context, encode

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    c.set_mixed_min_rows(0)
    yield c
    c.close()


def same_bits(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.array_equal(a.view(np.int64), b.view(np.int64)) or np.array_equal(a, b, equal_nan=True)


def check_plain(ds, ods, trees, tuned=True):
    b = encode(trees, tuned=tuned)
    dev, ora = ds.evaluate(b, PLAIN), ods.evaluate(b)
    assert np.array_equal(dev["size"], ora["size"])
    for key in ("loss", "rmse"):
        assert same_bits(dev[key], ora[key]), key
    return dev, ora


def test_empty_batch(ctx):
    X = np.random.default_rng(0).uniform(-1, 1, (100, 2))
    ds = ctx.dataset(X, X[:, 0] + X[:, 1])
    for prec in (PLAIN, MIXED, CERTIFIED):
        out = ds.evaluate(encode([], tuned=True), prec)
        assert len(out["loss"]) == 0
    ds.close()


@pytest.mark.parametrize("n", [1, 2, 3])
def test_tiny_datasets(ctx, n):
    rng = np.random.default_rng(n)
    X = rng.uniform(-2, 2, (n, 2))
    y = rng.uniform(-1, 1, n)
    ds, ods = ctx.dataset(X, y), pyoracle.OracleDataset(X, y)
    trees = ["x0", "add x0 x1", "mul x0 sin x1", "ln x0", "add mul c:2 x0 c:1"]
    check_plain(ds, ods, trees)
    check_plain(ds, ods, trees, tuned=False)
    # the mixed forms agree on the sentinel pattern
    ora = ods.evaluate(encode(trees, tuned=True))
    for prec in (MIXED, CERTIFIED):
        out = ds.evaluate(encode(trees, tuned=True), prec)
        assert np.array_equal(out["loss"] == 1000, ora["loss"] == 1000)
    ds.close()


def test_constant_target(ctx):
    # SST = 0: R2 is not finite, every candidate gets the sentinel or the
    # oracle's exact values
    rng = np.random.default_rng(3)
    X = rng.uniform(-2, 2, (5000, 3))
    y = np.full(5000, 1.5)
    ds, ods = ctx.dataset(X, y), pyoracle.OracleDataset(X, y)
    trees = ["x0", "add x0 x1", "sin x2", "mul x0 x1"]
    dev, ora = check_plain(ds, ods, trees)
    cert = ds.evaluate(encode(trees, tuned=True), CERTIFIED)
    assert np.array_equal(cert["loss"] == 1000, ora["loss"] == 1000)
    ds.close()


def test_untuned_candidates_in_mixed_forms(ctx):
    X, y, trees, _ = synth.batched_fitness(n=20_000, d=4, n_trees=200, seed=5)
    ds, ods = ctx.dataset(X, y), pyoracle.OracleDataset(X, y)
    b = encode(trees, tuned=False)
    ora = ods.evaluate(b, threads=8)
    ok = ora["loss"] != 1000
    fv = lambda r: (1 + r["loss"]) * (1 + r["rmse"]) * (1 + r["size"] * 1e-3)  # noqa: E731
    for prec in (MIXED, CERTIFIED):
        out = ds.evaluate(b, prec)
        assert np.array_equal(out["loss"] == 1000, ora["loss"] == 1000)
        assert np.array_equal(out["size"][ok], ora["size"][ok])
        err = np.abs(fv(out)[ok] - fv(ora)[ok]) / fv(ora)[ok]
        assert err.max() <= 1e-6
    ds.close()


def test_widest_qr_bucket_bit_exact(ctx):
    # 24 distinct factors plus the free term: more than 16 columns with y
    rng = np.random.default_rng(9)
    n = 70_000
    X = rng.uniform(-1.5, 1.5, (n, 3))
    y = np.sin(X[:, 0]) + X[:, 1] * X[:, 2] + 0.01 * rng.standard_normal(n)
    terms = []
    for i in range(3):
        terms += [f"x{i}", f"sin x{i}", f"cos x{i}", f"sqr x{i}"]
        terms += [f"exp mul c:{c} x{i}" for c in (0.1, 0.2, 0.3, 0.4)]
    tree = "add " * (len(terms) - 1) + " ".join(terms)
    trees = [tree] * 4 + [f"add {tree} mul x0 x1"]  # several, so the batch takes the shared table path
    trees += [synth.random_tree(rng, int(rng.integers(3, 12)), 3) for _ in range(400)]
    ds, ods = ctx.dataset(X, y), pyoracle.OracleDataset(X, y)
    b = encode(trees, tuned=True)
    assert b.cands[0]["n_factors"] >= 24
    dev, ora = ds.evaluate(b, PLAIN), ods.evaluate(b, threads=8)
    assert np.array_equal(dev["size"], ora["size"])
    for key in ("loss", "rmse", "rank"):
        assert same_bits(dev[key], ora[key]), key
    for i in range(5):
        assert same_bits(dev["coefs"][i], ora["coefs"][i])
    # scored alone (the one-block QR's single-candidate launch) the same bits
    alone = ds.evaluate(encode(trees[:1], tuned=True), PLAIN)
    for key in ("loss", "rmse", "rank"):
        assert same_bits(alone[key], dev[key][:1]), key
    ds.close()
