import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmfgpu.so")


@pytest.fixture(scope="session")
def ctx():
    import monofonic_gb300 as mf
    c = mf.Context(0)
    yield c
    # objects created by tests hold references to the context; it is
    # destroyed when the last of them is collected
