import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def gastar():
    """The engine package with libgastar.so built in-tree."""
    from cuda_a_star_gb300 import build
    build.build()
    import cuda_a_star_gb300 as g
    g.lib()
    return g


@pytest.fixture(scope="session")
def engine(gastar):
    e = gastar.Engine(0)
    yield e
    e.close()


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    oracle_lib.lib()
    return oracle_lib
