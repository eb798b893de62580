"""A whole search with the column cache on and off (rrh_set_column_cache):
the same model string, fit calls, rounds and predictions bit for bit, in the
plain FP64 drop-in and in the certified mixed form, on a dataset large enough
for the cache to be used."""
import numpy as np
import pytest

import rils_rols_cpp
from rils_rols_gb300 import synth

pytestmark = pytest.mark.gpu


def fit(X, y, precision, cache):
    n, d = X.shape
    m = rils_rols_cpp.rils_rols(False, 20000, 1 << 30, 0.001, 50, 1.0, False, 7)
    m.set_precision(precision)
    m.set_column_cache(cache)
    m.fit(X.reshape(-1), y, n, d)
    pred = m.predict(X.reshape(-1), n, d)
    return m.get_model_string(), m.get_fit_calls(), m.counters()["device_rounds"], pred


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_search_is_the_same_with_and_without_the_cache(precision):
    X, y = synth.regression_1m(n=30_000)
    on = fit(X, y, precision, True)
    off = fit(X, y, precision, False)
    assert on[0] == off[0]
    assert on[1] == off[1] and on[2] == off[2]
    assert np.array_equal(on[3], off[3])
