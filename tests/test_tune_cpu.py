"""Launch-shape tuner's host interface (no device work): the knobs and values
the kernels are built for, pins and the report (CPU only)."""
import pytest

from rils_rols_gb300 import _lib
from rils_rols_gb300.fitness import EVAL_WAVES, QR_WARPS, tune_mode, tune_pin, tune_report, tune_reset


@pytest.fixture(autouse=True)
def clean():
    tune_reset()
    yield
    tune_reset()
    tune_mode(True)


def test_pins_accept_built_shapes_only(lib):
    for bucket, shapes in ((4, (1, 2, 4)), (8, (2, 4, 8)), (16, (4, 8, 16)), (65, (8, 16))):
        for w in shapes:
            assert lib.rrg_tune_pin(QR_WARPS, bucket, w) == _lib.RRG_OK
        assert lib.rrg_tune_pin(QR_WARPS, bucket, 3) == _lib.RRG_E_INVALID
    assert lib.rrg_tune_pin(QR_WARPS, 5, 4) == _lib.RRG_E_INVALID
    assert lib.rrg_tune_pin(EVAL_WAVES, 0, 8) == _lib.RRG_OK
    assert lib.rrg_tune_pin(EVAL_WAVES, 0, 5) == _lib.RRG_E_INVALID
    assert lib.rrg_tune_pin(EVAL_WAVES, 1, 8) == _lib.RRG_E_INVALID
    assert lib.rrg_tune_pin(7, 0, 1) == _lib.RRG_E_INVALID
    assert b"not built" in lib.rrg_last_error() or b"unknown" in lib.rrg_last_error()
    assert lib.rrg_tune_set_mode(2) == _lib.RRG_E_INVALID


def test_report_lists_pins_and_reset_clears(lib):
    tune_pin(QR_WARPS, 8, 2)
    tune_pin(EVAL_WAVES, 0, 16)
    rep = tune_report()
    assert {"knob": "qr_warps", "bucket": 8, "pinned": 2} in rep
    assert {"knob": "eval_waves", "bucket": 0, "pinned": 16} in rep
    tune_pin(QR_WARPS, 8, 0)
    assert {"knob": "qr_warps", "bucket": 8, "pinned": 2} not in tune_report()
    tune_reset()
    assert tune_report() == []
    # the size query counts the terminating NUL
    assert lib.rrg_tune_report(None, 0) == 1
