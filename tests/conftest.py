import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")
    config.addinivalue_line("markers", "slow: longer statistical runs")


@pytest.fixture(scope="session")
def oracle():
    """The oracle's CPU library (built on first use)."""
    from tests import oracle_lib
    return oracle_lib.load()


@pytest.fixture(scope="session")
def native():
    """libjmmgpu.so, built in-tree if it is missing."""
    from jmmonedmc_gb300 import _native, build
    if not os.path.exists(_native.lib_path()):
        build.build_native()
    lib = _native.load()
    return lib


@pytest.fixture(scope="session")
def gpu(native):
    from jmmonedmc_gb300 import _native
    if not _native.device_available():
        pytest.fail("no CUDA device visible to libjmmgpu.so")
    return native
