import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (run with -m gpu)")


@pytest.fixture(scope="session")
def built_lib():
    """Builds libtfxgb300.so (incremental) and returns the ctypes handle."""
    from tressfx_gb300 import build as B
    B.build()
    from tressfx_gb300 import _capi
    return _capi.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    return oracle.lib()


@pytest.fixture(scope="session")
def ctx(built_lib):
    from tressfx_gb300.api import Context
    c = Context(int(os.environ.get("TFX_DEVICE", "0")))
    yield c
    c.close()
