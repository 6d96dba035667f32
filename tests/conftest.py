import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def built_lib():
    """Build (if needed) and load libfastkpm_gb300.so."""
    from fastkpm_gb300 import build
    build.build()
    from fastkpm_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(built_lib):
    import fastkpm_gb300 as fk
    if fk.device_count() == 0:
        pytest.fail("no CUDA device visible: the gpu tests need a GB300")
    return True


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def cheb_T(m, x):
    return np.cos(m * np.arccos(np.clip(x, -1, 1)))
