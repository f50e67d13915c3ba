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
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def engine():
    """Builds (if stale) and loads libluxum.so."""
    from luxum_gb300 import build as b

    b.build_library()
    from luxum_gb300 import _ffi

    return _ffi.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle

    return oracle.lib()
