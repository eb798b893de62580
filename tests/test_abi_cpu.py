"""The C-ABI library builds, loads and exports every symbol its headers declare;
argument checking needs no device."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

from rils_rols_gb300 import _lib

REPO = Path(__file__).resolve().parent.parent


def test_exports_every_declared_symbol(lib):
    declared = set()
    for h in ("rils_rols_gb300.h", "rils_rols_host.h", "rils_rols_serve.h"):
        text = (REPO / "include" / h).read_text()
        declared |= set(re.findall(r"\b(rr[ghs]_[a-z_]+)\s*\(", text))
    assert declared == set(_lib.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name


def test_abi_version(lib):
    assert lib.rrg_abi_version() == 1


def test_invalid_arguments_are_reported(lib):
    h = C.c_void_p()
    assert lib.rrg_dataset_create(None, None, None, 0, 0, C.byref(h)) == _lib.RRG_E_INVALID
    assert lib.rrg_round_wait(None, 0) == _lib.RRG_E_INVALID
    assert lib.rrg_context_destroy(None) == _lib.RRG_E_INVALID
    assert lib.rrh_fit(None, None, None, 0, 0) == _lib.RRG_E_INVALID
    assert b"invalid" in lib.rrh_last_error()


def test_encoder_output_is_well_formed():
    from rils_rols_gb300.fitness import encode
    b = encode(["add mul c:2 x0 sin x1", "x0", "c:3"], tuned=True)
    assert list(b.cands["n_factors"]) == [2, 1, 0]
    assert b.n_coefs == 3 + 2 + 1
    u = encode(["div x0 x1"], tuned=False)
    assert list(u.cands["n_factors"]) == [1] and u.n_coefs == 0
    # every program ends with EMIT of its last slot
    for c in b.cands:
        last = int(b.code[c["code_offset"] + c["code_len"] - 1])
        assert last & 0xFF == 11 and last >> 8 == max(c["n_factors"] - 1, 0) or c["n_factors"] == 0


def test_encoded_golden_batches_validate(golden, lib):
    from rils_rols_gb300.fitness import encode
    for name, spec in golden("fitness").items():
        d = len(spec["X"][0])
        trees = [c["tree"] for c in spec["cases"]]
        for tuned in (True, False):
            b = encode(trees, tuned=tuned)
            s = b.struct()
            assert lib.rrg_batch_validate(C.byref(s), d) == 0, (name, tuned, lib.rrg_last_error())
            if d > 1:  # a feature index beyond the dataset is refused
                assert lib.rrg_batch_validate(C.byref(s), 1) != 0 or all("x1" not in t for t in trees)


def test_validation_rejects_bad_code(lib):
    from rils_rols_gb300.fitness import encode
    b = encode(["add x0 sin x1"], tuned=False)
    b.code[0] = 0xFF  # unknown opcode
    s = b.struct()
    assert lib.rrg_batch_validate(C.byref(s), 2) == 1
