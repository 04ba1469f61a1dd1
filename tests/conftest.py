import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lt():
    """The product package; building it here if the library is missing."""
    try:
        import lighttraffic_gb300 as m
    except ImportError:
        from lighttraffic_gb300 import build as b  # noqa: F401  (package import fails first)
        raise
    return m


@pytest.fixture(scope="session")
def require_gpu():
    if not gpu_available():
        pytest.fail("this test is marked gpu but no CUDA device is visible")
