import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def built_lib():
    """Builds (if needed) and loads libmpsim_gb300.so."""
    import __graft_entry__ as g
    g.build()
    from mpsim_gb300 import _native
    return _native.load()


@pytest.fixture(scope="session")
def cuda(built_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device (no CPU fallback exists)"
    torch.cuda.set_device(0)
    return torch.device("cuda", 0)
