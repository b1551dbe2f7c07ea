import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libtay_gb300.so")


@pytest.fixture(scope="session")
def built():
    """Builds the engine library and the oracle (no-ops when up to date)."""
    from tay_gb300 import _build
    from oracle import pyoracle

    _build.build()
    pyoracle.build_port()
    return True


@pytest.fixture(scope="session")
def port(built):
    from oracle import pyoracle

    return pyoracle.port()


@pytest.fixture(scope="session")
def gpu(built):
    from tay_gb300 import api

    if api.lib().tgpu_device_count() == 0:
        pytest.fail("a GPU test ran without a visible CUDA device")
    return True
