import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libgraphyt_gpu.so")


@pytest.fixture(scope="session")
def oracle_built():
    """Build the CPU oracle (and the reference library where the reference tree exists)."""
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    from graphyt_gb300 import build, _lib
    build.build()
    return _lib.load()
