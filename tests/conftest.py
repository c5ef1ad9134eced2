import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def l1(a, b):
    """Relative L1 error per variable: sum|a-b| / sum|b| over all cells."""
    ax = tuple(range(a.ndim - 1))
    return np.abs(a - b).sum(axis=ax) / np.abs(b).sum(axis=ax)


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in place; fails loudly when it is missing."""
    from pypde_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from pypde_gb300 import build
        build.build()
    return _lib.lib()
