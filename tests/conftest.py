import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) CUDA device")


@pytest.fixture(scope="session")
def built():
    """Builds libuvatrmm.so and the oracle when missing (nvcc cross-compiles)."""
    from oracle import oracle
    from uvatrmm_gb300 import build

    build.build()
    oracle.build()
    return True


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def handle(built):
    if not gpu_available():
        pytest.skip("no CUDA device")
    import uvatrmm_gb300 as u
    return u.Handle()
