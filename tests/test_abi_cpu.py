"""C-ABI checks that need no GPU: the library loads, exports every function
declared in include/pisces_gb300.h, and its host-only entry points (kinetic
builder, water-site producer, rand() restatement) match the golden vectors."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden, rel


def header_functions():
    text = open(os.path.join(ROOT, "include", "pisces_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function(pg):
    lib = pg.lib()
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python front end declares the same set
    assert set(names) <= set(pg.SYMBOLS)


def test_status_and_version(pg):
    assert pg.lib().pg_version() >= 100
    # a bad argument is a status, not an exit
    x = np.empty(4)
    t = np.empty(10)
    s = pg.lib().pg_sine_dvr(0, 1.0, -1.0, 1.0, x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                             t.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0)
    assert s == pg.PG_BAD_ARG
    assert b"pg_sine_dvr" in pg.lib().pg_last_error()


def test_kinetic_builder_matches_reference(pg):
    g = golden("kinetic.npz")
    for key in g:
        if key.startswith("x_"):
            _, n, L = key.split("_")
            x, t = pg.sine_dvr(int(n), float(L))
            assert rel(x, g[key]) < 1e-15
            assert rel(t, g[f"t_{n}_{L}"]) < 1e-14
            # full storage (ldt = n) is the symmetric unpacking of the same numbers
            _, T = pg.sine_dvr(int(n), float(L), packed=False)
            a, b = np.tril_indices(int(n))
            assert np.array_equal(T[a, b], t) and np.array_equal(T, T.T)


@pytest.mark.parametrize("tag", ["w6", "w24"])
def test_water_site_producer_matches_reference(pg, tag):
    g = golden(f"dpp_{tag}.npz")
    t = pg.WaterTables(g["waters"])
    assert t.scf_iters > 0
    assert rel(t.sites, g["sites"]) < 1e-14
    assert np.array_equal(t.charges, g["charges"]) and np.array_equal(t.charge_site, g["charge_site"])
    assert np.array_equal(t.dipole_site, g["dipole_site"])
    assert rel(t.dipoles, g["dipoles"]) < 1e-11


def test_water_site_producer_rejects_nan(pg):
    w = np.zeros((1, 9))
    w[0, 4] = np.nan
    with pytest.raises(pg.PiscesError) as e:
        pg.WaterTables(w)
    assert e.value.status == pg.PG_BAD_ARG


def test_random_start_stream_is_c_library_rand(pg):
    libc = ctypes.CDLL(None)
    libc.srand(1)
    exp = [libc.rand() for _ in range(2000)]
    assert list(pg.glibc_rand_stream(2000)) == exp


@pytest.mark.parametrize("m,k", [(1, 1), (2, 1), (3, 2), (20, 4), (60, 4), (96, 16)])
def test_subspace_eigensolver(pg, m, k):
    rng = np.random.default_rng(m * 31 + k)
    A = rng.normal(size=(m, m))
    S = (A + A.T) / 2
    w, V = pg.subspace_lowest(np.triu(S), k)   # only the upper triangle is read
    wr = np.linalg.eigvalsh(S)[:k]
    assert np.max(np.abs(w - wr)) < 1e-12 * max(1.0, np.abs(wr).max())
    assert np.max(np.abs(S @ V - V * w)) < 1e-10
    assert np.max(np.abs(V.T @ V - np.eye(k))) < 1e-10


def test_subspace_eigensolver_degenerate(pg):
    # a cluster of equal eigenvalues (the box and harmonic spectra have them)
    rng = np.random.default_rng(2)
    Q, _ = np.linalg.qr(rng.normal(size=(30, 30)))
    lam = np.concatenate([[-1.0, 0.5, 0.5, 0.5, 0.5000001], np.linspace(1, 3, 25)])
    S = (Q * lam) @ Q.T
    w, V = pg.subspace_lowest(S, 5)
    assert np.max(np.abs(w - lam[:5])) < 1e-12
    assert np.max(np.abs(S @ V - V * w)) < 1e-10
    assert np.max(np.abs(V.T @ V - np.eye(5))) < 1e-10


def test_reference_shaped_header_compiles():
    """include/pisces_gb300_ref.hpp (the reference signatures over the C ABI)
    and its davdriver-style test driver compile as C++."""
    import shutil
    import subprocess
    cuda = "/usr/local/cuda/include"
    if not shutil.which("g++") or not os.path.isdir(cuda):
        pytest.skip("g++ or the CUDA headers are missing")
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), "-I", cuda,
                    os.path.join(ROOT, "tests", "shim", "check_ref_shim.cpp")], check=True)


def test_request_footprint_counts_the_solve_buffers(pg):
    # admission footprint (pg_request_footprint), in device bytes: basis and
    # products (2 maxsub N), the work array (2 nroots N for corrflag 1/3), the
    # diagonal, the potential, the eigenvectors (nroots N), the kinetic
    # preconditioner's blocks (7 nroots N, corrflag 3), the mixed form's
    # double-float twins of basis and products (2 maxsub N), and the small
    # subspace arrays (2 maxsub^2 + 11 maxsub)
    n, ms, nr = (48, 40, 56), 30, 3
    N = 48 * 40 * 56
    w = np.zeros((1, 9))
    def fp(**kw):
        return pg.Engine.footprint(pg.Engine.request(n, 20.0, w, nroots=nr, maxsub=ms, **kw))
    base = 8.0 * (N * (2 * ms + 2 * nr + 1 + 1 + nr) + 2 * ms * ms + 11 * ms)
    assert fp(corrflag=1, precision=pg.PG_FP64) == base
    assert fp(corrflag=3, precision=pg.PG_FP64) == base + 8.0 * N * 7 * nr
    assert fp(corrflag=3, precision=pg.PG_MIXED) == base + 8.0 * N * (7 * nr + 2 * ms)
