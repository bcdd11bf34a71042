import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def qvmlib():
    """The built C-ABI library (compiled here if missing)."""
    from qvm_gb300 import build
    from qvm_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.lib()


@pytest.fixture(scope="session")
def gpu():
    """Require a CUDA device; a missing library or device is an error, not a skip."""
    from qvm_gb300 import build
    build.build()
    import qvm_gb300
    info = qvm_gb300.device_info()
    assert info["sm_count"] > 0
    return info
