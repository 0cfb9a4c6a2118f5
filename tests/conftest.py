import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def bem():
    """The GPU package (built on first use; loading never falls back to CPU)."""
    mod = importlib.import_module("3d_bem_gb300")
    mod.build()
    return mod


@pytest.fixture(scope="session")
def meshes():
    return importlib.import_module("3d_bem_gb300.meshes")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
