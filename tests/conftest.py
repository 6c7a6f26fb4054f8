import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The autotuner's cache of this test session lives in a private temp file.
if "UVATRMM_TUNE_CACHE" not in os.environ:
    import tempfile
    os.environ["UVATRMM_TUNE_CACHE"] = os.path.join(tempfile.mkdtemp(prefix="uvatrmm_tune_"), "tune.txt")


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
