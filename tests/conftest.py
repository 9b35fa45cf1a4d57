import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs the engine's kernels")


@pytest.fixture(scope="session")
def goldens():
    return json.loads((GOLDEN / "reference_goldens.json").read_text())


@pytest.fixture(scope="session")
def O():
    from oracle import oracle

    oracle.build()
    return oracle
