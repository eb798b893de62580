"""Serving loop (csrc/host/serve.cpp) on the oracle backend: every job's model
is the reference's, alone and in a mix of concurrent jobs; admission follows
the device-memory footprint and the arrival order (CPU only)."""
import numpy as np
import pytest

from oracle import pyoracle
from rils_rols_gb300 import _lib
from rils_rols_gb300.serve import Server, ServeError

TOY = ["toy_3000_s0", "toy_3000_s1", "toy_3000_s7", "toy_sample_half"]


def _params(cfg):
    return dict(classification=bool(cfg["cls"]), max_fit_calls=cfg["max_fit_calls"], max_seconds=1 << 30,
                complexity_penalty=cfg["cp"], max_complexity=cfg["max_complexity"], sample_size=cfg["sample_size"],
                random_state=cfg["seed"])


def _data(fits):
    d = fits["toy_data"]
    return np.asarray(d["Xtr"]), np.asarray(d["ytr"])


def test_concurrent_jobs_match_reference(golden):
    fits = golden("fit")
    X, y = _data(fits)
    with Server(max_active=3, backend=pyoracle.backend_struct()) as srv:
        jobs = {key: srv.submit(X, y, **_params(fits[key]["cfg"])) for key in TOY}
        for key, job in jobs.items():
            model, info = srv.result(job)
            assert model == fits[key]["model"], key
            assert info["fit_calls"] == fits[key]["fit_calls"], key
            assert info["state"] == "done"
            assert info["time_to_model_s"] >= info["run_s"] > 0
        st = srv.stats()
    assert st["done"] == len(TOY) and st["failed"] == 0 and st["queued"] == 0
    assert 1 <= st["peak_running"] <= 3
    assert 0 < st["p50_time_to_model_s"] <= st["p99_time_to_model_s"]
    assert st["candidates"] > 0


def test_alone_equals_in_mix(golden):
    fits = golden("fit")
    X, y = _data(fits)
    key = "toy_3000_s1"
    with Server(max_active=1, backend=pyoracle.backend_struct()) as srv:
        alone, _ = srv.result(srv.submit(X, y, **_params(fits[key]["cfg"])))
    rng = np.random.default_rng(3)
    Xo = rng.uniform(-3, 3, (500, 3))
    yo = np.sin(Xo[:, 0]) * Xo[:, 1] + Xo[:, 2] ** 2
    with Server(max_active=4, backend=pyoracle.backend_struct()) as srv:
        others = [srv.submit(Xo, yo, max_fit_calls=3000, max_seconds=1 << 30, random_state=s) for s in range(3)]
        job = srv.submit(X, y, **_params(fits[key]["cfg"]))
        mixed, _ = srv.result(job)
        for o in others:
            srv.result(o)
        assert srv.stats()["peak_running"] >= 2
    assert mixed == alone == fits[key]["model"]


def test_admission_by_footprint(golden):
    fits = golden("fit")
    X, y = _data(fits)
    cfg = _params(fits["toy_3000_s0"]["cfg"])
    cfg["max_fit_calls"] = 2000
    with Server(max_active=4, backend=pyoracle.backend_struct(), memory_budget=1 << 40) as srv:
        probe = srv.submit(X, y, **cfg)
        srv.result(probe)
        fp = srv.info(probe)["footprint_bytes"]
    assert fp > 0
    # a budget for one job at a time: the jobs run one after another, in arrival order
    with Server(max_active=4, backend=pyoracle.backend_struct(), memory_budget=fp + fp // 2) as srv:
        jobs = [srv.submit(X, y, **dict(cfg, random_state=s)) for s in range(3)]
        infos = [srv.result(j)[1] for j in jobs]
        assert srv.stats()["peak_running"] == 1
    ends = [i["queued_s"] + i["run_s"] for i in infos]
    assert ends == sorted(ends)
    # a job larger than the whole budget is refused at submission
    with Server(max_active=2, backend=pyoracle.backend_struct(), memory_budget=fp // 2) as srv:
        with pytest.raises(ServeError, match="RRG_E_OOM"):
            srv.submit(X, y, **cfg)


def test_invalid_arguments(lib):
    assert not lib.rrs_create(0, 0, 0)
    assert b"invalid" in lib.rrs_last_error()
    with Server(max_active=1, backend=pyoracle.backend_struct()) as srv:
        with pytest.raises(ServeError):
            srv.submit(np.zeros((4, 2)), np.zeros(4), precision=7)
        with pytest.raises(ServeError):
            srv.result(12345)
    assert lib.rrs_set_backend(None, None) == _lib.RRG_E_INVALID


def test_bounded_bypass_of_a_blocked_head():
    # a budget for one large job and one small one: while the first large job
    # runs, the second (the head of the queue) does not fit, and the small jobs
    # behind it start first, but at most 8 of them pass it
    import time
    rng = np.random.default_rng(5)
    XL = rng.uniform(-2, 2, (40_000, 1))
    yL = np.sin(XL[:, 0]) + 0.5 * XL[:, 0]
    XS = rng.uniform(-2, 2, (300, 1))
    yS = XS[:, 0] ** 2 - XS[:, 0]
    with Server(max_active=4, backend=pyoracle.backend_struct(), memory_budget=1 << 40) as srv:
        fl = srv.info(srv.submit(XL, yL, max_fit_calls=50, max_seconds=1 << 30))["footprint_bytes"]
        fs = srv.info(srv.submit(XS, yS, max_fit_calls=50, max_seconds=1 << 30))["footprint_bytes"]
    assert fl > fs
    with Server(max_active=4, backend=pyoracle.backend_struct(), memory_budget=fl + fs + (fl - fs) // 2) as srv:
        t0 = time.perf_counter()
        submitted = {}
        l1 = srv.submit(XL, yL, max_fit_calls=3000, max_seconds=1 << 30, random_state=1)
        submitted[l1] = time.perf_counter() - t0
        l2 = srv.submit(XL, yL, max_fit_calls=200, max_seconds=1 << 30, random_state=2)
        submitted[l2] = time.perf_counter() - t0
        small = []
        for s in range(12):
            j = srv.submit(XS, yS, max_fit_calls=600, max_seconds=1 << 30, random_state=10 + s)
            submitted[j] = time.perf_counter() - t0
            small.append(j)
        infos = {j: srv.result(j)[1] for j in [l1, l2] + small}
    start = {j: submitted[j] + infos[j]["queued_s"] for j in infos}
    ahead = sum(start[j] < start[l2] for j in small)
    assert 1 <= ahead <= 8, ahead
    assert all(i["state"] == "done" for i in infos.values())
