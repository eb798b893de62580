"""Dataset upload on the device: X given row-major (rrg_dataset_create_rows,
transposed on the device) or column-major (rrg_dataset_create, one 2-D copy),
from pageable or pinned memory, gives the same resident data and so the same
bits in every precision; ragged row counts and one feature included."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle
from rils_rols_gb300 import synth
from rils_rols_gb300.fitness import CERTIFIED, MIXED, PLAIN, Context, encode

pytestmark = pytest.mark.gpu


def same(a, b):
    for k in ("loss", "rmse", "size", "rank", "flags"):
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    for ca, cb in zip(a["coefs"], b["coefs"]):
        assert np.array_equal(ca, cb, equal_nan=True)


@pytest.mark.parametrize("n,d", [(1000, 3), (4099, 1), (70001, 5)])
def test_row_and_column_uploads_agree(n, d):
    rng = np.random.default_rng(n)
    X = rng.uniform(-2, 2, (n, d))
    y = np.sin(X[:, 0]) + 0.5 * X[:, -1] ** 2 + 0.01 * rng.standard_normal(n)
    trees = [synth.random_tree(rng, int(rng.integers(3, 16)), d) for _ in range(60)]
    batch = encode(trees, tuned=True)
    ctx = Context(0)
    try:
        ds_rows = ctx.dataset(np.ascontiguousarray(X), y)          # row-major entry
        ds_cols = ctx.dataset(np.asfortranarray(X), y)             # column-major entry
        for prec in (PLAIN, MIXED, CERTIFIED):
            same(ds_rows.evaluate(batch, prec), ds_cols.evaluate(batch, prec))
        # pinned buffers through the C ABI directly
        lib = ctx.lib
        import torch
        Xp = torch.from_numpy(np.ascontiguousarray(X)).pin_memory().numpy()
        yp = torch.from_numpy(np.ascontiguousarray(y)).pin_memory().numpy()
        h = C.c_void_p()
        dp = C.POINTER(C.c_double)
        assert lib.rrg_dataset_create_rows(ctx.h, Xp.ctypes.data_as(dp), yp.ctypes.data_as(dp), n, d, C.byref(h)) == 0
        assert lib.rrg_dataset_rows(h) == n and lib.rrg_dataset_cols(h) == d
        lib.rrg_dataset_destroy(h)
        # the plain path against the oracle
        ora = pyoracle.OracleDataset(X, y).evaluate(batch)
        dev = ds_rows.evaluate(batch, PLAIN)
        ok = ora["loss"] != 1000
        assert np.array_equal(dev["size"], ora["size"])
        np.testing.assert_allclose(dev["loss"][ok], ora["loss"][ok], rtol=1e-10, atol=1e-300)
        ds_rows.close()
        ds_cols.close()
    finally:
        ctx.close()


def test_invalid_upload_arguments():
    ctx = Context(0)
    try:
        lib = ctx.lib
        h = C.c_void_p()
        y = np.zeros(4)
        dp = C.POINTER(C.c_double)
        assert lib.rrg_dataset_create_rows(ctx.h, None, y.ctypes.data_as(dp), 4, 2, C.byref(h)) != 0
        assert lib.rrg_dataset_create_rows(ctx.h, y.ctypes.data_as(dp), y.ctypes.data_as(dp), 0, 1, C.byref(h)) != 0
    finally:
        ctx.close()


def test_context_destroyed_before_its_datasets():
    """Garbage collection may finalise a context before the datasets that
    reference it (objects that die together are finalised in any order): the
    context then releases their device memory, the handles only accept
    rrg_dataset_destroy, and other calls on them fail cleanly."""
    from rils_rols_gb300._lib import RRGError
    rng = np.random.default_rng(11)
    X = rng.uniform(-1, 1, (5000, 2))
    y = X[:, 0] * 2.0 + X[:, 1]
    ctx = Context(0)
    ds_a = ctx.dataset(X, y)
    ds_b = ctx.dataset(X, y)
    batch = encode(["add x0 x1"], tuned=True)
    ref = ds_a.evaluate(batch, PLAIN)
    ds_b.close()  # the usual order for one of them
    ctx.close()   # the other outlives its context
    with pytest.raises(RRGError):
        ds_a.evaluate(batch, PLAIN)
    ds_a.close()
    # a fresh context works as before
    ctx2 = Context(0)
    try:
        ds = ctx2.dataset(X, y)
        same(ds.evaluate(batch, PLAIN), ref)
        ds.close()
    finally:
        ctx2.close()
