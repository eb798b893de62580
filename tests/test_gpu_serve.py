"""Serving loop on the device: concurrent jobs, each with its own context and
streams, give the reference's models (tests/golden/fit.json), and a job's
model in a mix equals its model alone, in FP64 and in the certified mixed
form."""
import numpy as np
import pytest

from rils_rols_gb300 import _lib
from rils_rols_gb300.serve import Server

pytestmark = pytest.mark.gpu

TOY = ["toy_3000_s0", "toy_3000_s1", "toy_3000_s7", "toy_sample_half"]


def _params(cfg, precision=_lib.RRG_PLAIN_FP64):
    return dict(classification=bool(cfg["cls"]), max_fit_calls=cfg["max_fit_calls"], max_seconds=1 << 30,
                complexity_penalty=cfg["cp"], max_complexity=cfg["max_complexity"], sample_size=cfg["sample_size"],
                random_state=cfg["seed"], precision=precision)


def test_concurrent_device_jobs_match_reference(golden):
    fits = golden("fit")
    X, y = np.asarray(fits["toy_data"]["Xtr"]), np.asarray(fits["toy_data"]["ytr"])
    cls = fits["cls_200x6"]
    with Server(max_active=4, memory_budget=64 << 30) as srv:
        jobs = {key: srv.submit(X, y, **_params(fits[key]["cfg"])) for key in TOY}
        jobs["cls_200x6"] = srv.submit(np.asarray(cls["X"]), np.asarray(cls["y"]), **_params(cls["cfg"]))
        for key, job in jobs.items():
            model, info = srv.result(job)
            assert model == fits[key]["model"], key
            assert info["fit_calls"] == fits[key]["fit_calls"], key
            assert info["device_rounds"] > 0
        st = srv.stats()
    assert st["done"] == len(jobs) and st["failed"] == 0
    assert st["peak_running"] >= 2


def test_certified_job_same_alone_and_in_mix(golden):
    fits = golden("fit")
    X, y = np.asarray(fits["toy_data"]["Xtr"]), np.asarray(fits["toy_data"]["ytr"])
    key = "toy_3000_s7"
    cfg = _params(fits[key]["cfg"], _lib.RRG_MIXED_CERTIFIED)
    with Server(max_active=1, memory_budget=16 << 30) as srv:
        alone, info_alone = srv.result(srv.submit(X, y, **cfg))
    rng = np.random.default_rng(5)
    Xo = rng.uniform(-3, 3, (20000, 4))
    yo = Xo[:, 0] * np.exp(0.3 * Xo[:, 1]) - np.cos(Xo[:, 2]) / (1.5 + Xo[:, 3] ** 2)
    with Server(max_active=4, memory_budget=64 << 30) as srv:
        others = [srv.submit(Xo, yo, max_fit_calls=20000, max_seconds=1 << 30, random_state=s,
                             precision=_lib.RRG_MIXED_CERTIFIED) for s in range(3)]
        mixed, info_mixed = srv.result(srv.submit(X, y, **cfg))
        for o in others:
            srv.result(o)
        assert srv.stats()["peak_running"] >= 2
    assert mixed == alone == fits[key]["model"]
    assert info_mixed["fit_calls"] == info_alone["fit_calls"]
