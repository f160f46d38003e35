import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def native_lib():
    """Build (if needed) and load the C-ABI library."""
    from bendy2d_gb300 import build as b
    b.build()
    from bendy2d_gb300 import _native
    return _native.load()


@pytest.fixture(scope="session")
def gpu(native_lib):
    if not HAS_GPU:
        pytest.skip("no CUDA device")
    return native_lib
