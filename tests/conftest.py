import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def lib():
    from final184_gb300 import build

    build.build()
    import final184_gb300

    return final184_gb300.load()


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.lib()
    return oracle
