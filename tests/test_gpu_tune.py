"""Launch-shape tuner on the device: every shape of a knob (FP64 evaluator
waves, and in mixed rounds the double-float evaluator's factors per block,
whether it stages X and y in shared memory by tensor copies, and the pair
sums' partners per block) gives the same bits, and the tuner times every
shape once per (knob, bucket, row class) and keeps the fastest."""
import numpy as np
import pytest

from oracle import pyoracle
from rils_rols_gb300.fitness import (CERTIFIED, EVAL_WAVES, FAC_GROUP, FAC_STAGE, MIXED, PAIR_UNIT, PLAIN, Context,
                                     encode, tune_mode, tune_pin, tune_report, tune_reset)

pytestmark = pytest.mark.gpu

TERMS = ["x0", "x1", "x2", "sin x0", "sin x1", "sin x2", "cos x0", "cos x1", "cos x2", "exp mul c:0.3 x0",
         "exp mul c:0.3 x1", "exp mul c:0.3 x2", "mul x0 x1", "mul x0 x2", "mul x1 x2", "sqr x0", "sqr x1", "sqr x2",
         "ln add c:4 x2", "div x0 add c:2 sqr x2", "mul x1 sin x2", "sqrt add c:5 x0", "cos mul x0 x2", "exp x1",
         "mul x0 cos x1"]


def sums(rng, count, lo, hi):
    out = []
    for _ in range(count):
        m = int(rng.integers(lo, hi + 1))
        t = [TERMS[i] for i in rng.choice(len(TERMS), m, replace=False)]
        out.append("add " * (m - 1) + " ".join(t))
    return out


@pytest.fixture(scope="module")
def data():
    rng = np.random.default_rng(11)
    n = 400_000
    X = rng.uniform(-2, 2, (n, 3))
    y = 1.5 * X[:, 0] * X[:, 1] - np.sin(X[:, 2]) + 0.1 * rng.standard_normal(n)
    # QR column buckets of k + 1 columns: <= 4 (1-2 terms), <= 8 (3-6), <= 16 (7-14)
    trees = sums(rng, 160, 1, 2) + sums(rng, 160, 3, 6) + sums(rng, 140, 7, 14)
    return X, y, trees


def same(a, b):
    for k in ("loss", "rmse", "size", "rank", "flags"):
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    for ca, cb in zip(a["coefs"], b["coefs"]):
        assert np.array_equal(ca, cb, equal_nan=True)


def test_every_shape_gives_the_same_bits(data):
    X, y, trees = data
    ctx = Context(0)
    ctx.set_column_cache(False)  # every round evaluates its columns: the shapes are timed and compared
    ds = ctx.dataset(X, y)
    batch = encode(trees, tuned=True)
    try:
        tune_mode(False)
        ref = ds.evaluate(batch, PLAIN)
        for wv in (2, 4, 8, 16):
            tune_pin(EVAL_WAVES, 0, wv)
            same(ds.evaluate(batch, PLAIN), ref)
        tune_pin(EVAL_WAVES, 0, 0)
        # and the oracle agrees bit for bit on a sample, scored alone and in the batch
        sub = encode(trees[::9], tuned=True)
        ora = pyoracle.OracleDataset(X, y).evaluate(sub)
        dev = ds.evaluate(sub, PLAIN)
        for k in ("loss", "rmse", "size", "rank"):
            assert np.array_equal(dev[k], ora[k], equal_nan=True), k
        idx = np.arange(0, len(trees), 9)
        assert np.array_equal(ref["loss"][idx], ora["loss"], equal_nan=True)
    finally:
        tune_reset()
        tune_mode(True)
        ds.close()
        ctx.close()


def test_tuner_times_every_shape_once(data):
    X, y, trees = data
    ctx = Context(0)
    ctx.set_column_cache(False)  # every round evaluates its columns: the shapes are timed and compared
    ds = ctx.dataset(X, y)
    batch = encode(trees, tuned=True)
    try:
        tune_mode(False)
        ref = ds.evaluate(batch, PLAIN)
        tune_reset()
        tune_mode(True)
        got = ds.evaluate(batch, PLAIN)
        same(got, ref)
        rep = {(e["knob"], e["bucket"]): e for e in tune_report()}
        rc = int(np.floor(np.log2(len(y))))
        e = rep[("eval_waves", 0)]
        assert e["row_class"] == rc
        assert set(e["ms"]) == {2, 4, 8, 16} and e["ms"][e["value"]] == min(e["ms"].values())
        # the choices stand: a second round times nothing new and gives the same bits
        before = tune_report()
        same(ds.evaluate(batch, PLAIN), ref)
        assert tune_report() == before
        # the certified mixed form runs its FP64 re-scoring through the same tuned launches
        cert = ds.evaluate(batch, CERTIFIED)
        assert np.array_equal(cert["size"], ref["size"])
    finally:
        tune_reset()
        ds.close()
        ctx.close()


def test_mixed_path_shapes_give_the_same_bits(data):
    X, y, trees = data
    ctx = Context(0)
    ctx.set_column_cache(False)  # every round evaluates its columns: the shapes are timed and compared
    ds = ctx.dataset(X, y)
    batch = encode(trees, tuned=True)
    try:
        tune_mode(False)
        for prec in (MIXED, CERTIFIED):
            ref = ds.evaluate(batch, prec)
            for g in (64, 32, 16):
                tune_pin(FAC_GROUP, 0, g)
                same(ds.evaluate(batch, prec), ref)
            tune_pin(FAC_GROUP, 0, 0)
            for u in (1 << 16, 512, 128):
                tune_pin(PAIR_UNIT, 0, u)
                same(ds.evaluate(batch, prec), ref)
            tune_pin(PAIR_UNIT, 0, 0)
            # X and y staged in shared memory by tensor copies, or read from L2
            for st in (2, 1):
                tune_pin(FAC_STAGE, X.shape[1], st)
                same(ds.evaluate(batch, prec), ref)
            tune_pin(FAC_STAGE, X.shape[1], 0)
        # with the tuner on, the first mixed round times both knobs' shapes
        # on its real launches and the results stay the same
        tune_reset()
        tune_mode(True)
        same(ds.evaluate(batch, CERTIFIED), ref)
        rep = {e["knob"]: e for e in tune_report()}
        assert set(rep["fac_group"]["ms"]) == {64, 32, 16}
        assert set(rep["pair_unit"]["ms"]) == {1 << 16, 512, 128}
        assert rep["pair_unit"]["ms"][rep["pair_unit"]["value"]] == min(rep["pair_unit"]["ms"].values())
        assert set(rep["fac_stage"]["ms"]) == {1, 2} and rep["fac_stage"]["bucket"] == X.shape[1]
    finally:
        tune_reset()
        tune_mode(True)
        ds.close()
        ctx.close()
