"""rrg_eval_plain_noalloc (fixed device scratch, no allocation) against
rrg_eval(RRG_PLAIN_FP64), called through the C ABI.

Each candidate is scored twice in a row by the allocation-free entry point
(the second call finds the first call's data still in the scratch) and once
by rrg_eval on a dataset holding the same X and y.  Both solve by the
direct column-pivoted QR in the same summation order (rrg_eval spreads
tall rows over the GPU, the allocation-free entry runs one block), so the
results are bit-identical at every row count.  The file sorts last so that
it also runs after every other test in the same process.
"""
import ctypes as C

import numpy as np
import pytest

from rils_rols_gb300 import _lib, synth
from rils_rols_gb300.fitness import PLAIN, Context, encode, result_dtype

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SCRATCH_BYTES = 32 << 20


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def trees_for(d, seed, count):
    rng = np.random.default_rng(seed)
    trees = [synth.random_tree(rng, int(rng.integers(1, 12)), d) for _ in range(count)]
    # a sum of several factors (multi-column OLS), a collinear pair, a
    # constant, a NaN producer and a tree with a repeated feature
    x2 = f"x{min(2, d - 1)}"
    trees += [f"add add mul c:2 x0 sin x1 add exp {x2} c:1.5",
              "add x0 mul c:3 x0",
              "c:4.25",
              "ln sub x0 c:100",
              f"add mul x1 x1 add cos x1 div {x2} c:7"]
    return trees


class DeviceData:
    """X (column-major, leading dimension ld) and y in device memory owned by the test."""

    def __init__(self, X, y, ld):
        n, d = X.shape
        Xcol = np.zeros((d, ld), dtype=np.float64)
        Xcol[:, :n] = X.T
        self.X = torch.from_numpy(Xcol).cuda()
        self.y = torch.from_numpy(np.ascontiguousarray(y, dtype=np.float64)).cuda()
        self.res = torch.zeros(result_dtype().itemsize, dtype=torch.uint8, device="cuda")
        self.coefs = torch.zeros(64, dtype=torch.float64, device="cuda")
        self.n, self.d, self.ld = n, d, ld
        torch.cuda.synchronize()

    def score(self, lib, batch):
        b = batch.struct()
        self.res.fill_(0xAB)  # stale bytes: the call must clear what it accumulates into
        self.coefs.fill_(-7.0)
        torch.cuda.synchronize()
        st = lib.rrg_eval_plain_noalloc(self.X.data_ptr(), self.ld, self.y.data_ptr(), self.n, self.d, C.byref(b),
                                        self.res.data_ptr(), self.coefs.data_ptr(), None)
        assert st == _lib.RRG_OK, _lib.last_error()
        res = self.res.cpu().numpy().view(result_dtype())[0]
        k = int(batch.cands[0]["n_factors"]) + 1 if batch.cands[0]["mode"] == _lib.RRG_TUNED else 0
        return res, self.coefs[:k].cpu().numpy().copy()


def same_result(a, b):
    for f in ("loss", "rmse", "size", "rank", "flags"):
        assert a[f] == b[f] or (np.isnan(a[f]) and np.isnan(b[f])), (f, a[f], b[f])


def check_against_eval(lib, ctx, X, y, trees, ld):
    dev = DeviceData(X, y, ld)
    ds = ctx.dataset(X, y)
    try:
        for tuned in (True, False):
            for t in trees:
                batch = encode([t], tuned=tuned)
                ref = ds.evaluate(batch, PLAIN)
                r1, c1 = dev.score(lib, batch)
                r2, c2 = dev.score(lib, batch)
                # two calls in a row agree bit for bit
                same_result(r1, r2)
                assert np.array_equal(c1, c2, equal_nan=True)
                for f in ("loss", "rmse", "size", "rank", "flags"):
                    a, b = r1[f], ref[f][0]
                    assert a == b or (np.isnan(a) and np.isnan(b)), (t, tuned, f, a, b)
                if tuned:
                    assert np.array_equal(c1, ref["coefs"][0], equal_nan=True), (t, c1, ref["coefs"][0])
    finally:
        ds.close()


def test_matches_plain_eval_direct(lib, ctx):
    rng = np.random.default_rng(7)
    n, d = 4096, 3
    X = rng.uniform(0.5, 4.0, size=(n, d))
    y = 2.0 * np.sin(X[:, 0]) + X[:, 1] * X[:, 2] - 0.5 + rng.normal(0, 0.01, n)
    # a leading dimension that is not a multiple of anything in particular
    check_against_eval(lib, ctx, X, y, trees_for(d, 11, 40), ld=n + 37)


def test_matches_plain_eval_ragged_small(lib, ctx):
    rng = np.random.default_rng(8)
    for n in (1, 2, 3, 255, 257):
        X = rng.uniform(-2.0, 2.0, size=(n, 2))
        y = X[:, 0] - 3.0 * X[:, 1] + 0.25
        check_against_eval(lib, ctx, X, y, trees_for(2, 100 + n, 6), ld=n)


def test_matches_plain_eval_tall(lib, ctx):
    rng = np.random.default_rng(9)
    n, d = 100_000, 3
    X = rng.uniform(0.5, 4.0, size=(n, d))
    y = np.exp(0.3 * X[:, 0]) + 2.0 * X[:, 1] - X[:, 2] + rng.normal(0, 0.05, n)
    trees = ["add add mul c:2 x0 sin x1 add exp x2 c:1.5", "add mul x0 x1 x2", "exp mul c:0.3 x0"]
    check_against_eval(lib, ctx, X, y, trees, ld=n)


def test_rejects_oversized_call_and_host_memory(lib):
    n = 2_000_000  # a 3-column OLS needs (2*3+1) * n * 8 = 112 MB > 32 MiB of scratch
    X = torch.zeros((2, n), dtype=torch.float64, device="cuda")
    y = torch.zeros(n, dtype=torch.float64, device="cuda")
    res = torch.zeros(result_dtype().itemsize, dtype=torch.uint8, device="cuda")
    coefs = torch.zeros(8, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    b = encode(["add x0 x1"], tuned=True).struct()
    st = lib.rrg_eval_plain_noalloc(X.data_ptr(), n, y.data_ptr(), n, 2, C.byref(b), res.data_ptr(),
                                    coefs.data_ptr(), None)
    assert st == _lib.RRG_E_TOO_LARGE
    assert "scratch" in _lib.last_error()
    assert 7 * n * 8 > SCRATCH_BYTES
    # host memory is refused before any launch
    Xh = np.zeros((2, 16))
    st = lib.rrg_eval_plain_noalloc(Xh.ctypes.data, 16, y.data_ptr(), 16, 2, C.byref(b), res.data_ptr(),
                                    coefs.data_ptr(), None)
    assert st == _lib.RRG_E_INVALID
    assert "device memory" in _lib.last_error()
