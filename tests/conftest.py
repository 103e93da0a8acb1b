import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libnbody_gb300.so (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(os.path.join(GOLDEN, name)))
    return load


@pytest.fixture(scope="session")
def nb():
    """The CUDA library; fails (does not skip) when it cannot run."""
    import nbody_gb300
    from nbody_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from nbody_gb300 import build
        build.build()
    _lib.load()
    return nbody_gb300
