import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libigr_gb300.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    if not os.path.exists(oracle_lib.LIB_PATH):
        oracle_lib.build()
    return oracle_lib


@pytest.fixture(scope="session")
def igr():
    import igr_sensitivities_gb300 as m
    from igr_sensitivities_gb300 import build
    if not os.path.exists(os.path.join(os.path.dirname(m.__file__), "libigr_gb300.so")):
        build.build()
    return m
