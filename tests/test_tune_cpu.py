"""Launch-shape tuner's host interface (no device work): the knobs and values
the kernels are built for, pins and the report (CPU only)."""
import pytest

from rils_rols_gb300 import _lib
from rils_rols_gb300.fitness import EVAL_WAVES, FAC_GROUP, FAC_STAGE, PAIR_UNIT, tune_mode, tune_pin, tune_report, tune_reset


@pytest.fixture(autouse=True)
def clean():
    tune_reset()
    yield
    tune_reset()
    tune_mode(True)


def test_pins_accept_built_shapes_only(lib):
    for knob, bucket, shapes in ((FAC_GROUP, 0, (64, 32, 16)), (PAIR_UNIT, 0, (65536, 512, 128)),
                                 (FAC_STAGE, 5, (1, 2)), (FAC_STAGE, 20, (1, 2))):
        for w in shapes:
            assert lib.rrg_tune_pin(knob, bucket, w) == _lib.RRG_OK
        assert lib.rrg_tune_pin(knob, bucket, 3) == _lib.RRG_E_INVALID
    assert lib.rrg_tune_pin(FAC_STAGE, 65, 1) == _lib.RRG_E_INVALID
    # the retired QR-shape knobs (0 and 5) take no pins
    assert lib.rrg_tune_pin(0, 8, 4) == _lib.RRG_E_INVALID
    assert lib.rrg_tune_pin(5, 8, 4) == _lib.RRG_E_INVALID
    assert lib.rrg_tune_pin(EVAL_WAVES, 0, 8) == _lib.RRG_OK
    assert lib.rrg_tune_pin(EVAL_WAVES, 0, 5) == _lib.RRG_E_INVALID
    assert lib.rrg_tune_pin(EVAL_WAVES, 1, 8) == _lib.RRG_E_INVALID
    assert lib.rrg_tune_pin(7, 0, 1) == _lib.RRG_E_INVALID
    assert b"not built" in lib.rrg_last_error() or b"unknown" in lib.rrg_last_error()
    assert lib.rrg_tune_set_mode(2) == _lib.RRG_E_INVALID


def test_report_lists_pins_and_reset_clears(lib):
    tune_pin(FAC_GROUP, 0, 32)
    tune_pin(EVAL_WAVES, 0, 16)
    rep = tune_report()
    assert {"knob": "fac_group", "bucket": 0, "pinned": 32} in rep
    assert {"knob": "eval_waves", "bucket": 0, "pinned": 16} in rep
    tune_pin(FAC_GROUP, 0, 0)
    assert {"knob": "fac_group", "bucket": 0, "pinned": 32} not in tune_report()
    tune_reset()
    assert tune_report() == []
    # the size query counts the terminating NUL
    assert lib.rrg_tune_report(None, 0) == 1
