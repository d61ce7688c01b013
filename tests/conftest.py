import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Builds the library, the scene source and the oracle once per session."""
    from bepuphysics1_gb300 import build
    import oracle
    build.build()
    oracle.build_oracle()
    yield


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_context():
    from bepuphysics1_gb300.solver import Context
    ctx = Context(int(os.environ.get("BEPUGPU_DEVICE", "0")))
    yield ctx
    ctx.close()
