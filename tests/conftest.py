import json
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "rils-rols_gb300"))
sys.path.insert(0, str(REPO))
GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) device")


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = json.loads((GOLDEN / f"{name}.json").read_text())
        return cache[name]

    return get


@pytest.fixture(scope="session")
def lib():
    from rils_rols_gb300 import _lib
    return _lib.load()
