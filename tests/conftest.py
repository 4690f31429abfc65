import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def qmc_lib():
    from rust_qmc_gb300 import build
    build.build()
    import rust_qmc_gb300 as Q
    return Q.load_library()


@pytest.fixture(scope="session")
def ctx(qmc_lib):
    import rust_qmc_gb300 as Q
    c = Q.Context(0)
    yield c
    c.close()
