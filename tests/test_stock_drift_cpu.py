"""How far the reference's own results move under stock arithmetic (the C
library's exp / log / sin / cos / pow and index-order sums, the reference's
setup.py flags) from the pinned arithmetic of the golden fixtures
(oracle/stock_drift.py).  Runs where the reference checkout was there to
build oracle/_ref/librr_ref_stock.so; measured on the golden sets: about 5%
of fitness triples differ by more than 1e-10 relative (almost all in the
rebuilt tree's size, a coefficient crossing the 1e-12 drop / snap rule),
no NaN sentinel changes, and five of the six golden fits keep their model
string (toy_100000 finds the same four terms in another order)."""
import pytest

from oracle import stock_drift

pytestmark = pytest.mark.skipif(not stock_drift.LIB.exists(), reason="stock reference build not present")


def test_stock_arithmetic_drift_is_bounded():
    rep = stock_drift.measure()
    total = sum(r["cases"] for r in rep["fitness"].values())
    differ = sum(r["differ"] for r in rep["fitness"].values())
    assert all(r["sentinel_changed"] == 0 for r in rep["fitness"].values())
    assert differ <= 0.1 * total, rep["fitness"]
    assert rep["fitness"]["tiny3x2"]["differ"] == 0
    fits = rep["fits"]
    assert all(f["fit_calls_same"] for f in fits.values()), fits
    assert sum(f["model_same"] for f in fits.values()) >= len(fits) - 1, fits
