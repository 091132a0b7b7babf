import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


_MESHES = {}


def icos(level: int, iters: int = 20):
    from tmcore_gb300 import mesh

    key = (level, iters)
    if key not in _MESHES:
        _MESHES[key] = mesh.generate_icos(level, iters)
    return _MESHES[key]


@pytest.fixture(scope="session")
def mesh3():
    return icos(3)


@pytest.fixture(scope="session")
def mesh4():
    return icos(4)


@pytest.fixture(scope="session")
def mesh5():
    return icos(5)


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library; GPU tests fail (not skip) when it cannot be used."""
    from tmcore_gb300 import _lib

    return _lib.gpu()


def rel_max(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
