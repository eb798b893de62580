"""The column-pivoted QR's rarely taken paths, bit for bit against the oracle,
in both device forms: one block per candidate (rows within one 16384-row
chunk) and the chunked passes over the GPU (more rows).  The candidates
exercise duplicate and constant factors (rank cuts), nearly collinear
factors (down-dated norms that must be recomputed), NaN and infinite
columns (NaN norms in the pivot scan), a reflector that is the identity,
and the widest column buckets; the certified form, whose re-scoring lane
runs the chunked passes from a device-decided list, must keep the oracle's
sentinels and sizes and stay within 1e-6."""
import numpy as np
import pytest

from oracle import pyoracle
from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import CERTIFIED, PLAIN, Context, encode

pytestmark = pytest.mark.gpu

TREES = [
    # duplicate factors, constant factors
    "add sin x0 add cos x1 sin x0",
    "add x0 add sin c:1 x1",
    "add mul x0 x1 add sin c:2 mul x1 x0",
    "add exp mul c:0.5 x2 add x3 exp mul c:0.5 x2",
    # nearly collinear factors: the norm down-dating loses accuracy
    "add x0 mul x0 add c:1 mul c:1e-9 x1",
    "add sin x2 add mul sin x2 add c:1 mul c:1e-7 x3 x0",
    "add x1 add mul x1 add c:1 mul c:1e-12 x0 mul x1 add c:1 mul c:2e-12 x2",
    # NaN and infinite columns
    "add ln x1 x0",
    "add x0 add sqrt x1 cos x2",
    "add exp mul c:800 x0 x1",
    "add x2 add ln sub x0 c:10 x3",
    "add div x0 sub x1 x1 x2",
    # a column of zeros (identity reflector)
    "add x0 mul c:0 x1",
]
# wide candidates: 10 and 17 distinct terms (QR buckets of 16 and 65 columns)
_T10 = ["x0", "x1", "x2", "x3", "sin x0", "sin x1", "sin x2", "sin x3", "cos x0", "cos x1"]
_T17 = ["mul x0 x1", "mul x1 x2", "mul x2 x3", "mul x3 x0", "exp mul c:0.1 x0", "exp mul c:0.1 x1", "sqr x2",
        "sqr x3", "div x0 add c:3 x1", "cos x3", "sin mul x0 x2", "ln add c:5 x2", "x0", "x1", "x2", "x3",
        "cos mul x1 x3"]
TREES += ["add " * (len(t) - 1) + " ".join(t) for t in (_T10, _T17)]


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    c.set_mixed_min_rows(0)
    yield c
    c.close()


def same_bits(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.all((a == b) | (np.isnan(a) & np.isnan(b)))


def data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-3, 3, (n, 4))
    y = 2.0 * X[:, 0] * X[:, 1] - np.sin(X[:, 2]) + 0.3 * np.exp(0.3 * X[:, 3]) + 0.01 * rng.standard_normal(n)
    trees = TREES + [synth.random_tree(rng, int(rng.integers(3, 25)), 4) for _ in range(150)]
    return X, y, trees


@pytest.mark.parametrize("n", [9000, 40000])
def test_plain_qr_paths_bit_exact(ctx, n):
    X, y, trees = data(n, 70 + n % 97)
    ds, ods = ctx.dataset(X, y), pyoracle.OracleDataset(X, y)
    b = encode(trees, tuned=True)
    dev, ora = ds.evaluate(b, PLAIN), ods.evaluate(b, threads=8)
    assert np.array_equal(dev["size"], ora["size"])
    assert np.array_equal(dev["rank"], ora["rank"])
    for key in ("loss", "rmse"):
        bad = np.flatnonzero(~((dev[key] == ora[key]) | (np.isnan(dev[key]) & np.isnan(ora[key]))))
        assert len(bad) == 0, (key, [trees[i] for i in bad[:3]])
    for i in range(len(trees)):
        assert same_bits(dev["coefs"][i], ora["coefs"][i]), trees[i]
    # each alone (the single-candidate launches of both forms): the same bits
    for i in range(len(TREES)):
        one = ds.evaluate(encode([trees[i]], tuned=True), PLAIN)
        assert same_bits(one["loss"], dev["loss"][i:i + 1]) and same_bits(one["coefs"][0], dev["coefs"][i]), trees[i]
    ds.close()


def test_certified_lane_on_hard_candidates(ctx):
    X, y, trees = data(40000, 5)
    ds, ods = ctx.dataset(X, y), pyoracle.OracleDataset(X, y)
    b = encode(trees, tuned=True)
    cert, ora = ds.evaluate(b, CERTIFIED), ods.evaluate(b, threads=8)
    assert ctx.last_round_stats()["fp64_rescored"] > 0
    sent = ora["loss"] == 1000
    assert np.array_equal(cert["loss"] == 1000, sent)
    assert np.array_equal(cert["size"][~sent], ora["size"][~sent])
    fv = lambda r: (1 + r["loss"]) * (1 + r["rmse"]) * (1 + 1e-3 * r["size"])  # noqa: E731
    ok = ~sent & np.isfinite(fv(ora))
    err = np.abs(fv(cert)[ok] - fv(ora)[ok]) / fv(ora)[ok]
    assert err.max() <= 1e-6
    ds.close()
