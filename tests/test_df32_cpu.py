"""Double-float arithmetic (rils-rols_gb300/csrc/common/df32.h) on the host:
accuracy against long-double references, and the special values the
evaluator relies on (NaN / inf with lo = 0, domain errors as in FP64)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
OPS = {"add": 0, "sub": 1, "mul": 2, "div": 3, "sqrt": 4, "exp": 5, "log": 6, "sin": 7, "cos": 8, "div_nc": 9}


@pytest.fixture(scope="module")
def df32(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("df32") / "df32_harness.so"
    subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                    str(HERE / "native" / "df32_harness.cpp"), "-o", str(out)], check=True)
    lib = C.CDLL(str(out))
    lib.df32_apply.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]

    def apply(op, a, b=None):
        a = np.ascontiguousarray(a, dtype=np.float64)
        out = np.empty_like(a)
        bb = None if b is None else np.ascontiguousarray(b, dtype=np.float64)
        lib.df32_apply(OPS[op], a.ctypes.data, None if bb is None else bb.ctypes.data, len(a), out.ctypes.data)
        return out
    return apply


def as_df(x):
    """The double-float value nearest to x (what the device holds)."""
    h = x.astype(np.float32).astype(np.float64)
    return h + (x - h).astype(np.float32).astype(np.float64)


def rel(x, ref):
    ref = np.asarray(ref, dtype=np.longdouble)
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1e-300)))


def test_basic_operations(df32):
    rng = np.random.default_rng(0)
    n = 100_000
    a = as_df(rng.uniform(-10, 10, n) * 10.0 ** rng.uniform(-5, 5, n))
    b = as_df(rng.uniform(-10, 10, n) * 10.0 ** rng.uniform(-5, 5, n))
    al, bl = a.astype(np.longdouble), b.astype(np.longdouble)
    assert rel(df32("add", a, b), al + bl) < 3e-14
    assert rel(df32("sub", a, b), al - bl) < 3e-14
    assert rel(df32("mul", a, b), al * bl) < 3e-14
    assert rel(df32("div", a, b), al / bl) < 6e-14
    # the evaluator's division: approximate reciprocal (here one ulp off) and
    # one Newton step; a zero divisor gives a non-finite leading part, which
    # sends the row to the guarded division
    assert rel(df32("div_nc", a, b), al / bl) < 6e-14
    z = df32("div_nc", np.array([1.0, 0.0, -2.0]), np.array([0.0, 0.0, 0.0]))
    assert not np.isfinite(z).any()
    assert rel(df32("sqrt", np.abs(a)), np.sqrt(np.abs(al))) < 3e-14


def test_elementary_functions(df32):
    rng = np.random.default_rng(1)
    n = 100_000
    x = as_df(rng.uniform(-60, 88, n))
    assert rel(df32("exp", x), np.exp(x.astype(np.longdouble))) < 5e-14
    # below about 1e-31 the low part leaves FP32's normal range: absolute accuracy only
    x = as_df(rng.uniform(-100, -60, n))
    assert float(np.max(np.abs(df32("exp", x) - np.exp(x.astype(np.longdouble))))) < 1e-38
    x = as_df(10.0 ** rng.uniform(-37, 38, n))
    err = np.abs(df32("log", x) - np.log(x.astype(np.longdouble)))
    assert float(err.max()) < 1e-12
    for name, f in (("sin", np.sin), ("cos", np.cos)):
        x = as_df(rng.uniform(-6000, 6000, n))
        err = np.abs(df32(name, x) - f(x.astype(np.longdouble)))
        assert float(err.max()) < 1e-13, name


def test_special_values(df32):
    nan, inf = np.nan, np.inf
    r = df32("log", np.array([0.0, -1.0, inf, nan]))
    assert r[0] == -inf and np.isnan(r[1]) and r[2] == inf and np.isnan(r[3])
    r = df32("exp", np.array([1000.0, -1000.0, nan]))
    assert r[0] == inf and r[1] == 0.0 and np.isnan(r[2])
    r = df32("div", np.array([1.0, 0.0, -1.0]), np.array([0.0, 0.0, 0.0]))
    assert r[0] == inf and np.isnan(r[1]) and r[2] == -inf
    r = df32("sqrt", np.array([-1.0, 0.0, inf]))
    assert np.isnan(r[0]) and r[1] == 0.0 and r[2] == inf
    # beyond the exact pi/2 reduction the value is reported as not computed
    assert np.isnan(df32("sin", np.array([1e6]))[0])
    r = df32("mul", np.array([inf, 3e38]), np.array([0.0, 3e38]))
    assert np.isnan(r[0]) and r[1] == inf
