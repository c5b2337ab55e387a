import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libwrfgpu.so")


@pytest.fixture(scope="session")
def gpulib():
    """The built CUDA library (GPU tests only)."""
    import ctypes
    from wrf_gb300 import gpu
    try:
        import torch  # noqa: F401 - only to confirm a device is visible
        have = torch.cuda.is_available()
    except Exception:
        have = True
    if not have:
        pytest.fail("no CUDA device visible for a test marked gpu")
    if not os.path.exists(gpu.lib_path()):
        import __graft_entry__ as g
        g.build()
    lib = gpu.load()
    assert isinstance(lib, ctypes.CDLL)
    return lib
