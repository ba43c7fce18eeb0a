import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build(ref=False)
    return O


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(os.path.join(GOLDEN, name)))
    return load


@pytest.fixture(scope="session")
def glib():
    """The built CUDA library (GPU tests only)."""
    from gmm_gb300 import build, _lib
    build.build()
    return _lib


@pytest.fixture()
def dev(glib):
    h = glib.Handle(0)
    yield h
    h.close()
