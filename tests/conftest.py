import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def gg():
    import accelgraph_express_gb300 as m

    if not os.path.exists(m.LIB_PATH):
        m.build()
    m.lib()
    return m


@pytest.fixture(scope="session")
def gpu(gg):
    """The product library with a device initialised; the GPU tests fail
    (not skip) when no device answers, so a silent CPU run cannot pass."""
    gg.device_init(0)
    return gg


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle_ctypes as O

    O.lib()
    return O
