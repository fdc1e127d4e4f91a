import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle_lib():
    from meep_gb300 import build
    return build.build_oracle()


@pytest.fixture(scope="session")
def engine_lib():
    from meep_gb300 import build
    return build.build_engine()


@pytest.fixture(scope="session")
def gpu_drivers():
    from meep_gb300 import build
    return build.build_drivers()
