import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libnxb_gb300.so")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    """Skips unless a GPU is present; returns the loaded product library."""
    if not _has_gpu():
        pytest.skip("no CUDA device")
    import nexusbvh_gb300 as nxb
    from nexusbvh_gb300 import _build
    _build.build_cuda()
    return nxb.load()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.load()
    return oracle
