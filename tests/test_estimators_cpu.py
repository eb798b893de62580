"""The scikit-learn style estimators (rils_rols package of this repository)
keep the reference's interface (rils_rols/rils_rols.py:16-190) and, with the
oracle as fitness backend, reproduce the reference's fits (CPU only)."""
import numpy as np
import pytest

from oracle import pyoracle
from rils_rols import RILSROLSBinaryClassifier, RILSROLSRegressor


def test_regressor_fit_matches_reference(golden):
    fits = golden("fit")
    data, case = fits["toy_data"], fits["toy_3000_s0"]
    cfg = case["cfg"]
    est = RILSROLSRegressor(max_fit_calls=cfg["max_fit_calls"], max_time=1 << 30, complexity_penalty=cfg["cp"],
                            max_complexity=cfg["max_complexity"], sample_size=cfg["sample_size"],
                            random_state=cfg["seed"])
    est.set_backend(pyoracle.backend_struct())
    X, y = np.asarray(data["Xtr"]), np.asarray(data["ytr"])
    assert est.fit(X, y) is est
    assert est.model == case["model"]
    assert est.fit_calls == case["fit_calls"]
    assert np.array_equal(est.predict(X), np.asarray(case["pred"]))
    r2 = est.score(X, y)
    assert 0.99 < r2 <= 1.0
    assert est.model_string() is not None
    report = est.fit_report_string()
    assert f"fitCalls={case['fit_calls']}" in report and case["model"] in report


def test_classifier_fit_matches_reference(golden):
    case = golden("fit")["cls_200x6"]
    cfg = case["cfg"]
    est = RILSROLSBinaryClassifier(max_fit_calls=cfg["max_fit_calls"], max_time=1 << 30,
                                   complexity_penalty=cfg["cp"], max_complexity=cfg["max_complexity"],
                                   sample_size=cfg["sample_size"], random_state=cfg["seed"])
    est.set_backend(pyoracle.backend_struct())
    X, y = np.asarray(case["X"]), np.asarray(case["y"])
    est.fit(X, y)
    assert est.model == case["model"]
    assert est.model_string() == case["model"]  # no simplification for classifiers
    pred = est.predict(X)
    assert np.array_equal(pred, (np.asarray(case["pred"]) > 0.5) * 1)
    p = est.predict_proba(X)
    assert p.shape == (len(X), 2) and np.allclose(p.sum(axis=1), 1.0)
    assert 0.0 <= est.score(X, y) <= 1.0


def test_interface_and_errors():
    est = RILSROLSRegressor(max_fit_calls=10, random_state=3)
    params = est.get_params()
    for k in ("max_fit_calls", "max_time", "complexity_penalty", "max_complexity", "sample_size", "verbose",
              "random_state"):
        assert k in params
    assert params["max_fit_calls"] == 10 and params["random_state"] == 3
    est.set_params(max_complexity=20)
    assert est.max_complexity == 20
    with pytest.raises(RuntimeError):
        est.predict(np.zeros((2, 2)))
    with pytest.raises(ValueError):
        RILSROLSRegressor(sample_size=1.5).fit(np.zeros((4, 2)), np.zeros(4))
    with pytest.raises(ValueError):
        RILSROLSBinaryClassifier().fit(np.zeros((4, 2)), np.array([0, 1, 2, 1]))
