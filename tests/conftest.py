import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the kernels")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build(reference=False)
    return oracle


@pytest.fixture(scope="session")
def cuda_lib():
    from graphaligner_gb300 import build
    build()
    from graphaligner_gb300._lib import lib
    return lib()
