import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def native():
    """The built native library (built in-tree on first use)."""
    from latticeflow_gb300 import _build
    _build.build_native()
    from latticeflow_gb300 import _native
    return _native.lib()


@pytest.fixture(scope="session")
def oracle_port():
    from oracle import oracle as O
    O.build_port()
    return O


@pytest.fixture(scope="session")
def gpu():
    import ctypes
    try:
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        rt = None
    try:
        import torch
        ok = torch.cuda.is_available()
    except Exception:
        ok = False
    if not ok:
        pytest.skip("no CUDA device")
    return True
