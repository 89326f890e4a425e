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


def dual_exact_mask(n, nc, xs, sites, rtol):
    """Points of an n^3 dual grid (nc coarse points per axis, coordinates xs
    per axis) whose V is evaluated exactly: not on a zeroed layer, not on
    the coarse lattice, and within rtol of some site
    (src/DVR.cpp:780-832)."""
    if n % 2 == 1:
        s, h, cut = 2, 0, n
    else:
        c = n - 3 * nc + 2
        s, h, cut = 3, c // 2, n - c
    p = np.arange(n) - h
    live = (p >= 0) & (p < cut)
    on = np.zeros(n, dtype=bool)
    on[live] = p[live] % s == 0
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    md = np.full(n ** 3, 50.0)
    for st in np.asarray(sites, dtype=np.float64).reshape(-1, 3):
        rx, ry, rz = xs[0][i] - st[0], xs[1][j] - st[1], xs[2][k] - st[2]
        md = np.minimum(md, np.sqrt(rx * rx + ry * ry + rz * rz))
    zero = ~(live[i] & live[j] & live[k])
    lattice = on[i] & on[j] & on[k]
    return ~zero & ~lattice & ~(md > rtol)
