import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built_lib():
    """Builds libodil_gb300.so if stale and returns its path."""
    from odil_gb300 import _build
    return _build.build()


@pytest.fixture(scope="session")
def cuda(built_lib):
    if not _has_gpu():
        pytest.fail("GPU test collected without a GPU")
    import torch
    torch.cuda.set_device(0)
    from odil_gb300 import _capi
    _capi.load()
    return torch.device("cuda:0")


@pytest.fixture(autouse=True)
def _drain_gpu_work(request):
    """A GPU test ends with its device work finished, so no kernel of one
    test still runs when the next one allocates (stream-ordered memory
    reuse across tests)."""
    yield
    if "cuda" in request.fixturenames:
        import torch
        torch.cuda.synchronize()
