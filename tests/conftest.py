import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built libfsig.so")


@pytest.fixture(scope="session")
def golden():
    import json
    return json.loads((GOLDEN / "ref_outputs.json").read_text())


@pytest.fixture(scope="session")
def engine():
    """One engine for the GPU tests.  There is no CPU fallback: a GPU test
    fails (not skips) when the engine cannot be created."""
    from fsig_gb300 import Engine
    e = Engine(0, arena_bytes=int(os.environ.get("FSIG_TEST_ARENA", 24 << 30)))
    yield e
    e.close()
