import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); parity tests through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Compile the library and the oracle once per session (fast when up to date)."""
    import __graft_entry__
    __graft_entry__.build()
    yield


@pytest.fixture(scope="session")
def gpu_ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without CUDA")
    from bsbolt_gb300 import extend
    ctx = extend.Context(0)
    yield ctx
    ctx.close()
