"""Full fits through the drop-in module with the device path: the same model
string and fitness-call count as the reference (tests/golden/fit.json)."""
import numpy as np
import pytest

import rils_rols_cpp

pytestmark = pytest.mark.gpu


def _fit(cfg, X, y, precision="plain"):
    m = rils_rols_cpp.rils_rols(bool(cfg["cls"]), cfg["max_fit_calls"], 1 << 30, cfg["cp"], cfg["max_complexity"],
                                cfg["sample_size"], False, cfg["seed"])
    m.set_precision(precision)
    X = np.asarray(X)
    m.fit(X.reshape(-1), np.asarray(y), X.shape[0], X.shape[1])
    return m


@pytest.mark.parametrize("key", ["toy_3000_s0", "toy_3000_s1", "toy_3000_s7", "toy_sample_half", "toy_100000"])
def test_device_fit_matches_reference(golden, key):
    fits = golden("fit")
    data, case = fits["toy_data"], fits[key]
    m = _fit(case["cfg"], data["Xtr"], data["ytr"])
    assert m.get_model_string() == case["model"]
    assert m.get_fit_calls() == case["fit_calls"]
    X = np.asarray(data["Xtr"])
    pred = m.predict(X.reshape(-1), X.shape[0], X.shape[1])
    np.testing.assert_allclose(pred, np.asarray(case["pred"]), rtol=1e-12, atol=1e-12)


def test_device_classifier_fit_matches_reference(golden):
    case = golden("fit")["cls_200x6"]
    m = _fit(case["cfg"], case["X"], case["y"])
    assert m.get_model_string() == case["model"]
    assert m.get_fit_calls() == case["fit_calls"]
