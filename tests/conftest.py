import os
import sys

import numpy as np
import pytest

# the oracle's OpenMP loops are small; more threads than this only contend
os.environ.setdefault("OMP_NUM_THREADS", "4")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (test infrastructure), built on first use."""
    mod = entry.load_oracle()
    mod.lib()
    return mod


@pytest.fixture(scope="session")
def pg():
    """The product package (libpisces_gb300.so must have been built)."""
    mod = entry.load_package()
    mod.lib()
    return mod


@pytest.fixture(scope="session")
def clusters():
    entry.load_package()
    import importlib
    return importlib.import_module("pisces_gb300.clusters")


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
