"""The portable FP64 elementary functions (rils-rols_gb300/csrc/common/rr_math.h)
on the host: error in ulps against 60-digit references over seeded inputs
spanning each function's range, and the special values of C's libm (CPU
only).  The device compiles the same source with round-to-nearest
intrinsics, and the GPU parity tests check it bit for bit against the oracle
built from it."""
import ctypes as C
import math
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")
mp.mp.dps = 60

HERE = Path(__file__).resolve().parent
OPS = {"exp": 0, "log": 1, "sin": 2, "cos": 3, "pow": 4}


@pytest.fixture(scope="module")
def rr(tmp_path_factory):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not available")
    out = tmp_path_factory.mktemp("rr") / "rr_math_harness.so"
    subprocess.run([gcc, "-std=c99", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                    str(HERE / "native" / "rr_math_harness.c"), "-o", str(out), "-lm"], check=True)
    lib = C.CDLL(str(out))
    lib.rr_apply.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]

    def apply(op, a, b=None):
        a = np.ascontiguousarray(a, dtype=np.float64)
        out = np.empty_like(a)
        bb = None if b is None else np.ascontiguousarray(b, dtype=np.float64)
        lib.rr_apply(OPS[op], a.ctypes.data, None if bb is None else bb.ctypes.data, len(a), out.ctypes.data)
        return out
    return apply


def ulp_err(got, exact):
    """|got - exact| in units of the last place of the double nearest exact."""
    out = []
    for g, e in zip(got, exact):
        if mp.isinf(e) or e == 0:
            out.append(0.0 if float(e) == g else np.inf)
            continue
        ed = float(e)
        if math.isinf(ed):
            out.append(0.0 if math.isinf(g) else np.inf)
            continue
        u = math.ulp(ed) if ed != 0 else 5e-324
        out.append(float(abs(mp.mpf(g) - e) / u))
    return np.array(out)


def test_exp_within_one_ulp(rr):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-1, 1, 3000), rng.uniform(-40, 40, 3000), rng.uniform(-745, 709.7, 2000),
                        rng.uniform(-1e-8, 1e-8, 500), np.array([0.0, 1e-300, -1e-300, 709.78, -708.5, -744.0])])
    got = rr("exp", x)
    err = ulp_err(got, [mp.exp(mp.mpf(v)) for v in x])
    assert err.max() <= 1.0, (err.max(), x[err.argmax()])
    assert np.mean(err) < 0.3


def test_log_within_one_ulp(rr):
    rng = np.random.default_rng(2)
    x = np.concatenate([np.exp(rng.uniform(-700, 700, 3000)), rng.uniform(0.5, 2.0, 3000),
                        1 + rng.uniform(-1e-3, 1e-3, 1000), 1 + rng.uniform(-1e-12, 1e-12, 300),
                        np.array([1.0, 0.7071067811865476, 1.4142135623730951, 1.4142135623730949, 2.0, 0.5,
                                  5e-324, 2.2250738585072014e-308, 1.7976931348623157e308])])
    got = rr("log", x)
    err = ulp_err(got, [mp.log(mp.mpf(v)) for v in x])
    assert err.max() <= 1.0, (err.max(), x[err.argmax()])
    assert np.mean(err) < 0.3


def test_sin_cos_within_two_ulp(rr):
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-4, 4, 3000), rng.uniform(-1e4, 1e4, 2000), rng.uniform(-1e18, 1e18, 500)])
    for op, fn in (("sin", mp.sin), ("cos", mp.cos)):
        got = rr(op, x)
        exact = [fn(mp.mpf(v)) for v in x]
        # absolute error near the zeros, in ulps of 1
        err = np.array([float(abs(mp.mpf(g) - e)) for g, e in zip(got, exact)]) / 2.0 ** -52
        rel_ok = ulp_err(got, exact) <= 2.0
        assert np.all(rel_ok | (err <= 1.0)), op


def test_pow_within_one_ulp(rr):
    rng = np.random.default_rng(4)
    a = np.exp(rng.uniform(-20, 20, 2000))
    b = rng.uniform(-10, 10, 2000)
    got = rr("pow", a, b)
    err = ulp_err(got, [mp.power(mp.mpf(p), mp.mpf(q)) for p, q in zip(a, b)])
    # exp(b log a) with log a and the product carried as double-doubles
    assert err.max() <= 1.0, (err.max(), a[err.argmax()], b[err.argmax()])


def test_special_values(rr):
    nan, inf = float("nan"), float("inf")
    e = rr("exp", np.array([nan, inf, -inf, 710.0, -746.0, 0.0]))
    assert np.isnan(e[0]) and e[1] == inf and e[2] == 0.0 and e[3] == inf and e[4] == 0.0 and e[5] == 1.0
    lg = rr("log", np.array([nan, -1.0, 0.0, -0.0, inf, 1.0]))
    assert np.isnan(lg[0]) and np.isnan(lg[1]) and lg[2] == -inf and lg[3] == -inf and lg[4] == inf and lg[5] == 0.0
    s = rr("sin", np.array([nan, inf, -inf, 0.0, -0.0]))
    assert np.isnan(s[:3]).all() and s[3] == 0.0 and math.copysign(1, s[4]) == -1
    p = rr("pow", np.array([-8.0, -8.0, 0.0, 2.0, 1.0, nan]), np.array([1 / 3, 3.0, -1.0, 0.0, nan, 0.0]))
    assert np.isnan(p[0]) and p[1] == -512.0 and p[2] == inf and p[3] == 1.0 and p[4] == 1.0 and p[5] == 1.0
