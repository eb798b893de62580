"""The host search driver (csrc/host/search.cpp) reproduces the reference's
full fits when its fitness backend is the oracle (CPU only)."""
import numpy as np
import pytest

import rils_rols_cpp
from oracle import pyoracle


def _fit(cfg, X, y):
    m = rils_rols_cpp.rils_rols(bool(cfg["cls"]), cfg["max_fit_calls"], 1 << 30, cfg["cp"], cfg["max_complexity"],
                                cfg["sample_size"], False, cfg["seed"])
    m.set_backend(pyoracle.backend_struct())
    X = np.asarray(X)
    m.fit(X.reshape(-1), np.asarray(y), X.shape[0], X.shape[1])
    return m


@pytest.mark.parametrize("key", ["toy_3000_s0", "toy_3000_s1", "toy_3000_s7", "toy_sample_half", "toy_100000"])
def test_toy_fits_match_reference(golden, key):
    fits = golden("fit")
    data = fits["toy_data"]
    case = fits[key]
    m = _fit(case["cfg"], data["Xtr"], data["ytr"])
    assert m.get_model_string() == case["model"]
    assert m.get_model_prefix() == case["prefix"]
    assert m.get_fit_calls() == case["fit_calls"]
    X = np.asarray(data["Xtr"])
    pred = m.predict(X.reshape(-1), X.shape[0], X.shape[1])
    assert np.array_equal(pred, np.asarray(case["pred"]))


def test_classifier_fit_matches_reference(golden):
    case = golden("fit")["cls_200x6"]
    m = _fit(case["cfg"], case["X"], case["y"])
    assert m.get_model_string() == case["model"]
    assert m.get_fit_calls() == case["fit_calls"]
    X = np.asarray(case["X"])
    pred = m.predict(X.reshape(-1), X.shape[0], X.shape[1])
    # the golden holds the raw values of predict_inner; predict binarizes at 0.5 (rils_rols_cpp.cpp:744-745)
    assert np.array_equal(pred, (np.asarray(case["pred"]) >= 0.5) * 1.0)


def test_bad_sizes_raise_instead_of_exit():
    m = rils_rols_cpp.rils_rols(False, 100, 10, 0.001, 50, 1.0, False, 0)
    with pytest.raises(ValueError):
        m.fit(np.zeros(5), np.zeros(2), 2, 2)
