"""Shared test setup: the `gpu` marker, repository import path, oracle build."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build(ref=True)
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library; GPU tests fail loudly when it is missing."""
    import rajzel_gb300 as R
    R.load_library()
    return R
