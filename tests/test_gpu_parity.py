"""Device fitness path against the oracle and the reference's golden vectors.

Plain FP64 (one block per candidate while the rows fit one chunk, the
chunked passes beyond): bit-identical to the oracle, which is bit-identical
to the reference built with the same reduction order.  Mixed: penalised
fitness within the tolerances below of the FP64 oracle.
"""
import numpy as np
import pytest

from oracle import pyoracle
from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import CERTIFIED, MIXED, PLAIN, Context, encode

pytestmark = pytest.mark.gpu

REL_PLAIN = 1e-10


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    c.set_mixed_min_rows(0)  # the mixed kernels on every dataset size
    yield c
    c.close()


def test_small_datasets_take_fp64_in_mixed_rounds():
    # below the row threshold a mixed or certified round is the FP64 round,
    # bit for bit; at threshold 0 the mixed kernels run (within tolerance)
    rng = np.random.default_rng(4)
    n = 3000
    X = rng.uniform(-3, 3, (n, 3))
    y = X[:, 0] * np.exp(0.3 * X[:, 1]) - np.cos(X[:, 2])
    trees = [synth.random_tree(rng, int(rng.integers(3, 20)), 3) for _ in range(80)]
    b = encode(trees, tuned=True)
    c = Context(0)
    try:
        ds = c.dataset(X, y)
        plain = ds.evaluate(b, PLAIN)
        for prec in (MIXED, CERTIFIED):
            got = ds.evaluate(b, prec)
            for key in ("loss", "rmse", "size", "rank"):
                assert np.array_equal(got[key], plain[key], equal_nan=True), key
        launches_fp64 = c.last_round_launches()
        c.set_mixed_min_rows(0)
        cert = ds.evaluate(b, CERTIFIED)
        assert c.last_round_launches() != launches_fp64
        ok = plain["loss"] != 1000
        np.testing.assert_allclose(fitness_value(cert["loss"], cert["rmse"], cert["size"])[ok],
                                   fitness_value(plain["loss"], plain["rmse"], plain["size"])[ok], rtol=1e-6)
        ds.close()
    finally:
        c.close()


def rel_err(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    both_inf = np.isinf(a) & np.isinf(b) & (np.sign(a) == np.sign(b))
    err = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    err[both_inf] = 0.0
    err[(a == b)] = 0.0
    return err


def fitness_value(loss, rmse, size, cp=0.001):
    return (1 + np.asarray(loss)) * (1 + np.asarray(rmse)) * (1 + np.asarray(size) * cp)


def check_plain(dev, ora, tag):
    assert np.array_equal(dev["size"], ora["size"]), tag
    sent_d, sent_o = dev["loss"] == 1000, ora["loss"] == 1000
    assert np.array_equal(sent_d, sent_o), tag
    ok = ~sent_o
    # 1 - R2 is compared through R2 itself (1 - R2 == 0 for exact fits)
    assert np.all(rel_err(1 - dev["loss"][ok], 1 - ora["loss"][ok]) <= REL_PLAIN), tag
    assert np.all(rel_err(dev["rmse"][ok], ora["rmse"][ok]) <= REL_PLAIN + 1e-300), tag


def same_bits(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.all((a == b) | (np.isnan(a) & np.isnan(b)))


@pytest.mark.parametrize("name", ["toy", "rand257x3", "cls120x4", "tiny3x2"])
def test_plain_bit_exact_with_golden(ctx, golden, name):
    spec = golden("fitness")[name]
    X, y = np.array(spec["X"]), np.array(spec["y"])
    ds = ctx.dataset(X, y)
    ods = pyoracle.OracleDataset(X, y)
    trees = [c["tree"] for c in spec["cases"]]
    for tuned in (True, False):
        b = encode(trees, tuned=tuned)
        dev, ora = ds.evaluate(b, PLAIN), ods.evaluate(b)
        key = "tuned" if tuned else "untuned"
        gold = np.array([c[key]["fit"] for c in spec["cases"]], dtype=np.float64)
        assert same_bits(dev["loss"], gold[:, 0]), (name, tuned)
        assert same_bits(dev["rmse"], gold[:, 1]), (name, tuned)
        assert np.array_equal(dev["size"], gold[:, 2].astype(int)), (name, tuned)
        assert same_bits(dev["loss"], ora["loss"]) and same_bits(dev["rmse"], ora["rmse"])
        if tuned:
            for i in range(len(trees)):
                assert same_bits(dev["coefs"][i], ora["coefs"][i]), trees[i]


def test_plain_tall_few_candidates_bit_exact(ctx):
    # tall rows, few candidates: the chunked QR passes spread each candidate
    # over the GPU in the oracle's summation order
    X, y, trees, _ = synth.batched_fitness(n=100_000, d=5, n_trees=24, seed=3, max_size=25)
    ds = ctx.dataset(X, y)
    ods = pyoracle.OracleDataset(X, y)
    b = encode(trees, tuned=True)
    dev, ora = ds.evaluate(b, PLAIN), ods.evaluate(b, threads=8)
    check_plain(dev, ora, "tall")
    for f in ("loss", "rmse", "rank"):
        assert same_bits(dev[f], ora[f]), f
    for i in range(len(trees)):
        assert same_bits(dev["coefs"][i], ora["coefs"][i]), trees[i]


def test_plain_batched_medium_bit_exact(ctx):
    X, y, trees, _ = synth.batched_fitness(n=40_000, d=4, n_trees=400, seed=5, max_size=40)
    ds = ctx.dataset(X, y)
    ods = pyoracle.OracleDataset(X, y)
    for tuned in (True, False):
        b = encode(trees, tuned=tuned)
        dev, ora = ds.evaluate(b, PLAIN), ods.evaluate(b, threads=8)
        assert same_bits(dev["loss"], ora["loss"]) and same_bits(dev["rmse"], ora["rmse"]), tuned
        assert np.array_equal(dev["size"], ora["size"])


def test_predict_matches_oracle(ctx):
    X, y, trees, _ = synth.batched_fitness(n=5000, d=3, n_trees=20, seed=9)
    ds = ctx.dataset(X, y)
    ods = pyoracle.OracleDataset(X, y)
    for t in trees:
        got = ds.predict(t)
        want = ods.predict(encode([t], tuned=False))
        assert same_bits(got, want), t


@pytest.mark.parametrize("n,d,seed", [(20_000, 6, 13), (3000, 3, 4), (300, 2, 5)])
def test_mixed_certified_against_fp64_oracle(ctx, n, d, seed):
    # every mixed fitness within 1e-6 relative of the FP64 oracle (the
    # certification re-scores in FP64 whatever it cannot bound), the same NaN
    # sentinels, the same best candidate
    X, y, trees, _ = synth.batched_fitness(n=n, d=d, n_trees=600, seed=seed)
    ds = ctx.dataset(X, y)
    ods = pyoracle.OracleDataset(X, y)
    for tuned in (True, False):
        b = encode(trees, tuned=tuned)
        mix, ora = ds.evaluate(b, CERTIFIED), ods.evaluate(b, threads=8)
        assert np.array_equal(mix["loss"] == 1000, ora["loss"] == 1000), tuned
        assert np.array_equal(mix["size"], ora["size"]), tuned
        ok = ora["loss"] != 1000
        fv_m = fitness_value(mix["loss"], mix["rmse"], mix["size"])[ok]
        fv_o = fitness_value(ora["loss"], ora["rmse"], ora["size"])[ok]
        err = rel_err(fv_m, fv_o)
        assert np.all(err <= 1e-6), (tuned, float(err.max()))
        best = lambda r: int(np.argmin(np.where(ok, fitness_value(r["loss"], r["rmse"], r["size"]), np.inf)))  # noqa
        assert best(mix) == best(ora), tuned


def test_mixed_uncertified_close_to_fp64(ctx):
    # the fast mixed form: same NaN sentinels, most fitnesses within 1e-6
    X, y, trees, _ = synth.batched_fitness(n=20_000, d=6, n_trees=600, seed=13)
    ds = ctx.dataset(X, y)
    b = encode(trees, tuned=True)
    mix, ora = ds.evaluate(b, MIXED), pyoracle.OracleDataset(X, y).evaluate(b, threads=8)
    assert np.array_equal(mix["loss"] == 1000, ora["loss"] == 1000)
    ok = ora["loss"] != 1000
    err = rel_err(fitness_value(mix["loss"], mix["rmse"], mix["size"])[ok],
                  fitness_value(ora["loss"], ora["rmse"], ora["size"])[ok])
    # rank cuts (pivoted Cholesky) and the drop / snap rules may decide
    # differently from the FP64 QR for exactly collinear factor sets
    assert np.median(err) <= 1e-8 and np.mean(err <= 1e-6) >= 0.75


def test_round_is_deterministic_and_mix_independent(ctx):
    # the same candidate scores bit-identically alone and inside a larger batch
    X, y, trees, _ = synth.batched_fitness(n=8192, d=4, n_trees=300, seed=21)
    ds = ctx.dataset(X, y)
    for prec in (PLAIN, MIXED, CERTIFIED):
        full = ds.evaluate(encode(trees, tuned=True), prec)
        for i in (0, 17, 299):
            one = ds.evaluate(encode([trees[i]], tuned=True), prec)
            assert one["loss"][0] == full["loss"][i] or (np.isnan(one["loss"][0]) and np.isnan(full["loss"][i]))
            assert one["rmse"][0] == full["rmse"][i] or (np.isnan(one["rmse"][0]) and np.isnan(full["rmse"][i]))


def test_nonfinite_outcomes_decided_from_column_statistics(ctx):
    # Infinite and NaN factor values in various columns: where a column norm
    # is non-finite the QR's outcome (all-NaN coefficients at full rank) is
    # decided without running it; every result stays bit-identical to the
    # oracle, whether decided or factorised.
    rng = np.random.default_rng(11)
    n = 3000
    X = rng.uniform(-3, 3, (n, 3))
    y = 2.0 * X[:, 0] * X[:, 1] + np.sin(X[:, 2])
    X[5, 0] = 800.0    # exp(x0) overflows on one row
    X[17, 2] = -0.5    # x2 stays mixed-sign: ln and sqrt give NaN on part of the rows
    trees = ["add mul c:2 exp x0 mul c:3 x1", "add mul c:2 x1 mul c:3 exp x0",
             "add mul c:2 ln x2 mul c:3 x1", "add mul c:2 x1 mul c:3 ln x2",
             "add add mul c:2 x1 mul c:3 x0 mul c:4 sqrt x2", "add add mul c:2 sqrt x2 mul c:3 x0 exp x0",
             "add add add mul c:2 x1 mul c:3 x0 mul c:4 sin x2 ln x2", "add mul c:2 x1 mul c:3 x0",
             "mul exp x0 ln x2", "add exp mul c:1000 x1 x0"]
    ds = ctx.dataset(X, y)
    ods = pyoracle.OracleDataset(X, y)
    b = encode(trees, tuned=True)
    dev, ora = ds.evaluate(b, PLAIN), ods.evaluate(b)
    stats = ctx.last_round_stats()
    for key in ("loss", "rmse", "rank"):
        assert same_bits(dev[key], ora[key]), key
    assert np.array_equal(dev["size"], ora["size"])
    for i in range(len(trees)):
        assert same_bits(dev["coefs"][i], ora["coefs"][i]), trees[i]
    n_sent = int((ora["loss"] == 1000).sum())
    assert 1 <= stats["qr_skipped_sentinel"] <= n_sent
