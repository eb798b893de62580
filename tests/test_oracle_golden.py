"""The oracle (oracle/rrg_oracle.c) against the reference's own tune_constants
and fitness (golden vectors of tests/golden/fitness.json): bit-exact."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle
from rils_rols_gb300.fitness import encode

BUF = C.create_string_buffer(1 << 20)


@pytest.mark.parametrize("name", ["toy", "rand257x3", "cls120x4", "tiny3x2"])
def test_oracle_matches_reference(golden, lib, name):
    ds_spec = golden("fitness")[name]
    X, y = np.array(ds_spec["X"]), np.array(ds_spec["y"])
    ods = pyoracle.OracleDataset(X, y)
    trees = [c["tree"] for c in ds_spec["cases"]]
    for tuned, key in ((True, "tuned"), (False, "untuned")):
        batch = encode(trees, tuned=tuned)
        out = ods.evaluate(batch)
        for i, case in enumerate(ds_spec["cases"]):
            want = case[key]["fit"]
            got = [out["loss"][i], out["rmse"][i], int(out["size"][i])]
            assert got == want, (name, key, case["tree"], got, want)
            if tuned:
                coefs = np.ascontiguousarray(out["coefs"][i])
                r = lib.rrh_rebuild(case["tree"].encode(), coefs.ctypes.data_as(C.POINTER(C.c_double)), len(coefs),
                                    BUF, len(BUF))
                assert r >= 0
                model, prefix = BUF.value.decode().split("\t")
                # the sign of a NaN coefficient depends on operand order inside
                # the compiled arithmetic, not on the algorithm
                unsign = lambda t: t.replace("-nan", "nan")  # noqa: E731
                assert unsign(model) == unsign(case[key]["model"]), (case["tree"], model)
                assert unsign(prefix) == unsign(case[key]["prefix"]), (case["tree"], prefix)


def test_oracle_threads_do_not_change_results(golden):
    spec = golden("fitness")["rand257x3"]
    X, y = np.array(spec["X"]), np.array(spec["y"])
    ods = pyoracle.OracleDataset(X, y)
    batch = encode([c["tree"] for c in spec["cases"]], tuned=True)
    a, b = ods.evaluate(batch, threads=1), ods.evaluate(batch, threads=4)
    assert np.array_equal(a["loss"], b["loss"]) and np.array_equal(a["rmse"], b["rmse"])


def test_sentinel_on_nan():
    X = np.array([[-1.0], [-2.0], [-3.0]])
    y = np.array([1.0, 2.0, 4.0])
    out = pyoracle.OracleDataset(X, y).evaluate(encode(["ln x0"], tuned=False))
    assert (out["loss"][0], out["rmse"][0], out["size"][0]) == (1000.0, 1000.0, 1000)
