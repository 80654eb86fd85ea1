import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libsdgpu.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle.pyoracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def ref_oracle():
    from oracle import build
    if build.build_ref() is None and not os.path.exists(build.REF_SO):
        pytest.skip("reference sources not present: oracle/_ref cannot be built here")
    from oracle.pyoracle import Oracle
    return Oracle(ref=True)


@pytest.fixture(scope="session")
def gpu():
    from backends import GpuBackend
    return GpuBackend()
