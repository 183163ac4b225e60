"""Shared test set-up: import paths, the `gpu` marker, the oracle build."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "ader-dg_gb300"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    import pyoracle
    pyoracle.build()
    yield


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built if needed; GPU tests fail loudly without it."""
    import aderdg
    aderdg.build()
    return aderdg.load()
