import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "lattie-boltzmann-method-note_of_paperreview_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def islbm_lib():
    """The CUDA library, built in-tree if needed (nvcc cross-compiles without a GPU)."""
    import islbm_build as pkg_build
    pkg_build.build()
    import islbm
    islbm.load()
    return islbm


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import build as ob
    ob.build()
    from oracle import oracle
    return oracle


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.sqrt(np.sum(b * b))
    return float(np.sqrt(np.sum((a - b) ** 2)) / (den if den > 0 else 1.0))
