"""Bounded waits (rrg_round_wait with a timeout) on a round that is still on
the GPU: the wait returns RRG_E_TIMEOUT and leaves the round in flight, the
context refuses a second round meanwhile (RRG_E_INVALID), and an unbounded
wait then completes it with the results a blocking rrg_eval gives.  The wait
is on the host only: nothing on the GPU waits for anything."""
import ctypes as C
import gzip

import numpy as np
import pytest

from rils_rols_gb300 import _lib, synth
from rils_rols_gb300.fitness import CERTIFIED, PLAIN, Context, encode, result_dtype

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def rounds_1m():
    trees = [line.split("\t")[1] for line in gzip.open(GOLDEN / "ls_rounds_regression_1m.txt.gz", "rt")
             .read().splitlines()]
    return trees


@pytest.mark.parametrize("precision", [PLAIN, CERTIFIED])
def test_wait_times_out_then_completes(precision):
    X, y = synth.regression_1m()
    ctx = Context(0)
    try:
        ds = ctx.dataset(X, y)
        b = encode(rounds_1m(), tuned=True)
        want = ds.evaluate(b, precision)  # also settles the launch-shape tuner's trials
        lib = ctx.lib
        res = np.zeros(len(b), dtype=result_dtype())
        coefs = np.zeros(max(1, b.n_coefs))
        s = b.struct()
        st = lib.rrg_round_submit(ds.h, C.byref(s), precision, res.ctypes.data_as(C.POINTER(_lib.Result)),
                                  coefs.ctypes.data_as(C.POINTER(C.c_double)))
        assert st == _lib.RRG_OK, _lib.last_error()
        assert lib.rrg_round_wait(ctx.h, 0) == _lib.RRG_E_TIMEOUT
        # one round in flight per context
        res2 = np.zeros(len(b), dtype=result_dtype())
        st2 = lib.rrg_round_submit(ds.h, C.byref(s), precision, res2.ctypes.data_as(C.POINTER(_lib.Result)),
                                   coefs.ctypes.data_as(C.POINTER(C.c_double)))
        assert st2 == _lib.RRG_E_INVALID
        assert lib.rrg_round_wait(ctx.h, -1) == _lib.RRG_OK
        for f in ("loss", "rmse", "size", "rank", "flags"):
            assert np.array_equal(res[f], want[f], equal_nan=True), f
        # the context is usable afterwards
        again = ds.evaluate(b, precision)
        assert np.array_equal(again["loss"], want["loss"], equal_nan=True)
        ds.close()
    finally:
        ctx.close()
