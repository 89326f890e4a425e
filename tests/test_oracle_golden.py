"""CPU oracle pinned against golden vectors from the reference CPU code.

The fixtures in tests/golden/ were produced by the reference PISCES code built
from its own sources (tests/golden/make_golden.py).  These tests run on the
CPU only and check the oracle restatement that the GPU parity tests use as
their checker.
"""
import numpy as np
import pytest

from conftest import golden, rel


def test_kinetic_matrices_match_reference(orc):
    g = golden("kinetic.npz")
    for key in g:
        if not key.startswith("x_"):
            continue
        _, n, L = key.split("_")
        x, t = orc.sine_dvr(int(n), float(L))
        assert np.array_equal(x, g[key]) or rel(x, g[key]) < 1e-15
        assert rel(t, g[f"t_{n}_{L}"]) < 1e-14


def test_empty_box_spectrum_is_particle_in_a_box(orc):
    # The sine DVR is the DVR of the box eigenfunctions: T_axis has the exact
    # eigenvalues (pi k / L)^2 / 2 (src/sine_dvr.cpp:1-12).
    for n, L in [(16, 20.0), (33, 31.0)]:
        x, tp = orc.sine_dvr(n, L)
        w = np.linalg.eigvalsh(orc.unpack(tp, n))
        k = np.arange(1, n + 1)
        exact = (3.14159265358979 * k / L) ** 2 / 2
        assert np.max(np.abs(w - exact) / exact) < 1e-12


@pytest.mark.parametrize("tag", ["w6", "w24"])
def test_water_sites_match_reference(orc, tag):
    g = golden(f"dpp_{tag}.npz")
    sites, q, qs, d, ds, it = orc.dpp_sites(g["waters"])
    assert it > 0
    assert rel(sites, g["sites"]) < 1e-14
    assert np.array_equal(q, g["charges"]) and np.array_equal(qs, g["charge_site"])
    assert np.array_equal(ds, g["dipole_site"])
    assert rel(d, g["dipoles"]) < 1e-11


@pytest.mark.parametrize("tag", ["w6", "w24"])
def test_potential_matches_reference(orc, tag):
    g = golden(f"dpp_{tag}.npz")
    grid = orc.Grid(g["n"], g["L"])
    v, pc, ind, rep, pol = grid.potential_dpp(g["sites"], g["charges"], g["charge_site"], g["dipoles"],
                                              g["dipole_site"], parts=True)
    assert rel(v, g["v"]) < 1e-14
    for a, k in [(pc, "v_pc"), (ind, "v_ind"), (rep, "v_rep"), (pol, "v_pol")]:
        assert rel(a, g[k]) < 1e-14, k
    assert rel(grid.diagonal(g["v"]), g["diag"]) < 1e-15


@pytest.mark.parametrize("name", ["dpp_w6.npz", "dpp_w24.npz", "small_w6.npz", "ions_small.npz"])
def test_matvec_matches_reference(orc, name):
    g = golden(name)
    grid = orc.Grid(g["n"], g["L"])
    assert rel(grid.matvec(g["v"], g["mv_x"]), g["mv_y"]) < 1e-13


def test_ions_potential_matches_reference(orc):
    g = golden("ions_small.npz")
    grid = orc.Grid(g["n"], g["L"])
    sites, q, qs, d, ds, _ = orc.dpp_sites(g["waters"])
    v = grid.potential_dpp(sites, q, qs, d, ds)
    grid.add_ions(v, g["ion_sites"], g["ion_charges"])
    assert rel(v, g["v"]) < 1e-13


def test_davidson_two_states_match_reference(orc):
    g = golden("small_w6.npz")
    grid = orc.Grid(g["n"], g["L"])
    st, ev, vec, nmv = grid.solve(g["v"], nstates=2, ptol=8)
    assert st == 2
    assert np.max(np.abs(ev - g["evals"])) < 1e-10
    W = g["wavefn"].reshape(2, -1)
    for r in range(2):
        ov = abs(vec[r] @ W[r]) / np.linalg.norm(vec[r]) / np.linalg.norm(W[r])
        assert ov > 1 - 1e-10


def test_davidson_c1_matches_reference(orc):
    # (H2O)6, 32^3 sine grid over 30 bohr, lowest state, plain FP64 Davidson
    g = golden("c1.npz")
    grid = orc.Grid(g["n"], g["L"])
    sites, q, qs, d, ds, _ = orc.dpp_sites(g["waters"])
    v = grid.potential_dpp(sites, q, qs, d, ds)
    assert rel(v[g["v_idx"]], g["v_at"]) < 1e-14
    assert abs(v.sum() - g["v_sum"]) < 1e-9 * abs(g["v_sum"])
    st, ev, vec, nmv = grid.solve(v, nstates=1, ptol=8)
    assert st == 1
    assert abs(ev[0] - g["evals"][0]) < 1e-8
    w = g["wavefn32"].astype(np.float64)
    assert abs(vec[0] @ w) / np.linalg.norm(vec[0]) / np.linalg.norm(w) > 1 - 1e-8


def test_analytic_cases(orc):
    g = golden("analytic.npz")
    # empty box: the ground level is the sum of three 1-D box levels
    grid = orc.Grid(g["box_n"], g["box_L"])
    st, ev, _, _ = grid.solve(np.zeros(grid.N), nstates=1, ptol=8)
    exact = sum((3.14159265358979 / L) ** 2 / 2 for L in g["box_L"])
    assert st == 1 and abs(ev[0] - exact) < 1e-9
    assert abs(ev[0] - g["box1_evals"][0]) < 1e-10
    # three box states: the reference stops at its macro-iteration limit with
    # one converged root and leaves the eigenvalues unset; so does the oracle
    st, ev, _, _ = grid.solve(np.zeros(grid.N), nstates=3, ptol=8)
    assert st == int(g["box_nconv"][0]) == 1
    assert np.array_equal(ev, g["box_evals"])
    # harmonic well 0.5 k r^2: E0 -> 1.5 sqrt(k) (src/Model_pot.cpp:149)
    grid = orc.Grid(g["harm_n"], g["harm_L"])
    st, ev, _, _ = grid.solve(grid.spherical(float(g["harm_k"])), nstates=1, ptol=8)
    assert abs(ev[0] - g["harm_evals"][0]) < 1e-9
    assert abs(ev[0] - 1.5 * np.sqrt(float(g["harm_k"]))) < 1e-4
    # dense diagonalisation of a <= 1000-point water-cluster Hamiltonian
    grid = orc.Grid(g["full_n"], g["full_L"])
    st, ev, _, _ = grid.solve(g["full_v"], nstates=3, ptol=8, maxsub=40)
    assert st == 3
    assert np.max(np.abs(ev - g["full_evals"][:3])) < 1e-9
    assert np.max(np.abs(ev - g["full_dav_evals"])) < 1e-10


def test_start_vectors_random_stream_is_c_library_rand(orc):
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand(1)
    seq = [libc.rand() for _ in range(50)]
    # the oracle's Randm11 draws come from the same stream
    libc.srand(1)
    out = (ctypes.c_double * 5)()
    orc.lib().or_random_start.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    orc.lib().or_random_start(5, out)
    libc.srand(1)
    exp = []
    for _ in range(5):
        s = libc.rand()
        m = libc.rand()
        exp.append(m / 2147483647 if s > 2147483647 // 2 else -m / 2147483647)
    assert np.allclose(list(out), exp, rtol=0, atol=0)
    assert len(set(seq)) > 40


# ---------------------------------------------------------------- FFT kinetic path

def test_fft_kinetic_builder_matches_tdiag_restatement(orc, pg):
    """pg_fft_kinetic (host) against the numpy restatement of Tdiag: the same
    points and plane-wave energies, and its circulant matrix is the operator
    ifft(ekin fft(.)) / n of one axis (applied to unit vectors)."""
    for n, L in ((12, 9.0), (15, 11.0), (32, 30.0)):
        x, e, t = pg.fft_kinetic(n, L)
        xo, eo = orc.fft_tdiag(n, 1.0, -0.5 * L, 0.5 * L)
        assert np.array_equal(x, xo)
        assert np.allclose(e, eo, rtol=1e-15, atol=0)
        eye = np.eye(n)
        cols = np.real(np.fft.ifft(eo[:, None] * np.fft.fft(eye, axis=0), axis=0))
        assert np.max(np.abs(t - cols)) <= 1e-13 * np.max(np.abs(t))


@pytest.mark.parametrize("n", [12, 13])
def test_fft_path_matches_reference_run(orc, pg, n):
    """The FFT kinetic path against the reference run (fft.npz: DVR::SetupDVR
    with DVRType 3 and VectorFFT::apply on seeded vectors, cubic grids of even
    and odd size, FFTW replaced by the DFT from its definition in the oracle
    build): the restated grid points, Tdiag energies and KE_diag bit for bit,
    the library's host builder's points and energies likewise, and the
    restated VectorFFT::apply within 1e-14 of the largest |y| (the transforms
    sum in another order)."""
    g = golden("fft.npz")
    L = float(g[f"L_{n}"][0])
    for a in range(3):
        xo, eo = orc.fft_tdiag(n, 1.0, -0.5 * L, 0.5 * L)
        assert np.array_equal(xo, g[f"x{a}_{n}"])
        assert np.array_equal(eo, g[f"ekin{a}_{n}"])
        x, e, _ = pg.fft_kinetic(n, L)
        assert np.array_equal(x, g[f"x{a}_{n}"])
        assert np.array_equal(e, g[f"ekin{a}_{n}"])
    ke = orc.fft_ke_diag((n, n, n), (L, L, L))
    assert np.array_equal(ke, g[f"ke_diag_{n}"])
    for rep in range(2):
        y = orc.fft_apply(g[f"fft_x{rep}_{n}"], g[f"fft_v_{n}"], (n, n, n), ke)
        ref = g[f"fft_y{rep}_{n}"]
        assert np.max(np.abs(y - ref)) <= 1e-14 * np.max(np.abs(ref))


def test_fft_apply_is_three_axis_circulants(orc, pg):
    """The reference's 3-D FFT matvec equals V x plus the per-axis circulant
    contractions (cubic grid, where the reference's KE_diag indexing is
    consistent): the form the GPU kernels apply."""
    n, L = 10, 8.0
    rng = np.random.Generator(np.random.PCG64(3))
    x = rng.standard_normal(n ** 3)
    v = rng.standard_normal(n ** 3)
    y = orc.fft_apply(x, v, (n, n, n), orc.fft_ke_diag((n, n, n), (L, L, L)))
    _, _, t = pg.fft_kinetic(n, L)
    X = x.reshape(n, n, n)  # [k][j][i], x fastest
    ref = v * x + (np.einsum("ab,kjb->kja", t, X) + np.einsum("ab,kbi->kai", t, X)
                   + np.einsum("ab,bji->aji", t, X)).reshape(-1)
    assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))



def test_oracle_is_deterministic_across_thread_counts(orc):
    # the oracle's dot products sum fixed blocks in a fixed order, so a solve
    # gives the same bits whatever OpenMP thread count runs it
    import os
    import subprocess
    import sys
    from conftest import ROOT
    script = (
        "import sys, numpy as np\n"
        f"sys.path.insert(0, {ROOT!r})\n"
        "import __graft_entry__ as e\n"
        "orc = e.load_oracle()\n"
        f"g = dict(np.load({os.path.join(ROOT, 'tests', 'golden', 'small_w6.npz')!r}))\n"
        "st, ev, vec, nmv = orc.Grid(g['n'], g['L']).solve(g['v'], nstates=2, ptol=8)\n"
        "print(st, nmv, ev.tobytes().hex(), vec.tobytes()[:4096].hex())\n")
    outs = []
    for threads in ("1", "3"):
        env = dict(os.environ, OMP_NUM_THREADS=threads)
        r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        outs.append(r.stdout)
    assert outs[0] == outs[1]
