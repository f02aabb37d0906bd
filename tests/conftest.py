import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU and the built libmars_gpu.so (runs on the GB300)")


@pytest.fixture(scope="session")
def port():
    """The C restatement of the reference CPU path (built on first use)."""
    import oracle

    if not oracle.available("port"):
        oracle.build(with_reference=False)
    return oracle.load("port")


@pytest.fixture(scope="session")
def port_lib(port):
    import oracle

    return oracle.marslib_for("port")


@pytest.fixture(scope="session")
def built_lib():
    """Path of libmars_gpu.so, compiling it if it is missing."""
    from mars_gb300 import build, marslib

    if not os.path.isfile(marslib.LIB_PATH):
        build.build()
    return marslib.LIB_PATH


@pytest.fixture(scope="session")
def gpu(built_lib):
    """The marslib module, with a visible CUDA device."""
    from mars_gb300 import marslib

    marslib.load()
    assert marslib.device_count() > 0, "gpu tests need a visible CUDA device"
    return marslib
