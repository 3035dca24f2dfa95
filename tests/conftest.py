import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle_lib():
    from alens_gb300 import oracle_api
    return oracle_api.load_oracle()


@pytest.fixture(scope="session")
def gpu_lib():
    from alens_gb300 import build, capi
    build.build_lib()
    return capi.load_library()
