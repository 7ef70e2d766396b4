import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"
# the reference checkout (x86 container only; absent on the GPU host)
REFERENCE = Path(os.environ.get("BLPG_REFERENCE", "/root/reference"))
NETLIB = GOLDEN / "netlib"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def built():
    """libblpg.so and the oracle, built in-tree (no-op when up to date)."""
    from simplexprojects_gb300 import build as B
    B.build_all()
    return True


@pytest.fixture(scope="session")
def workloads_golden():
    p = GOLDEN / "workloads.json"
    if not p.exists():
        pytest.skip("tests/golden/workloads.json not generated")
    return json.loads(p.read_text())


@pytest.fixture(scope="session")
def known_golden():
    p = GOLDEN / "known.json"
    if not p.exists():
        pytest.skip("tests/golden/known.json not generated")
    return json.loads(p.read_text())


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
