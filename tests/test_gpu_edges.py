"""Edge cases of the device path against the CPU oracle.

  - the smallest and ragged grids (n = 2 on an axis, odd sizes, one long axis):
    H*X in FP64 and split-TF32 against the oracle's matvec (Hamiltonian::matvec,
    src/Hamiltonian.cpp), where the tensor-core tiles are mostly padding;
  - an empty block (nvec = 0) is a no-op that succeeds;
  - the largest root count one solve takes (16 roots in a 128-vector subspace)
    against the dense eigenvalues of the full Hamiltonian built column by column
    from the oracle, on well separated and on near-degenerate spectra, which
    the reference algorithm does not finish (its restart lets locked and new
    Ritz vectors drift apart from orthonormality);
  - the kinetic preconditioner outside its domain reports PG_NOT_CONVERGED;
  - a cluster with no waters is the particle in a box;
  - argument limits (roots, subspace, grid sizes) are PG_BAD_ARG before any
    launch, and the library keeps working after a rejected call.
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

MIXED_HX_TOL = 2e-5  # split-TF32 products, FP32 accumulation (same bound as the parity tests)


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def dev(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def host(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("n", [(2, 2, 2), (3, 5, 7), (2, 17, 9), (129, 2, 3), (5, 3, 130)])
def test_hx_tiny_and_ragged_grids(pg, orc, torch, n):
    L = tuple(0.6 * (k + 1) for k in n)
    rng = np.random.default_rng(sum(n))
    grid = pg.Grid(n, L)
    og = orc.Grid(n, L)
    nvec = 3
    v = rng.normal(size=grid.N)
    X = rng.normal(size=(nvec, grid.N))
    ref = np.stack([og.matvec(v, X[r]) for r in range(nvec)])
    y64 = host(grid.hx(dev(torch, v), dev(torch, X), precision=pg.PG_FP64)).reshape(nvec, -1)
    assert rel(y64, ref) < 1e-13
    ymx = host(grid.hx(dev(torch, v), dev(torch, X), precision=pg.PG_MIXED)).reshape(nvec, -1)
    assert np.max(np.abs(ymx - ref)) / np.max(np.abs(ref)) < MIXED_HX_TOL


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_hx_empty_block(pg, torch, precision):
    grid = pg.Grid((8, 8, 8), (6.0, 6.0, 6.0))
    v = torch.zeros(grid.N, dtype=torch.float64, device="cuda")
    X = torch.zeros(0, dtype=torch.float64, device="cuda")
    Y = torch.full((4,), 7.0, dtype=torch.float64, device="cuda")
    grid.hx(v, X, nvec=0, precision=precision, out=Y)
    assert float(Y.sum()) == 28.0  # nothing written


def _dense_h(og, v):
    N = og.N
    H = np.empty((N, N))
    e = np.zeros(N)
    for j in range(N):
        e[j] = 1.0
        H[:, j] = og.matvec(v, e)
        e[j] = 0.0
    return H


def _well(n, L, seed):
    """A confining well with a little noise: 8x7x9 has well separated
    levels; on 12x11x13 boxes of near-equal sides its p- and d-like levels are
    split by 5e-4 Eh only."""
    rng = np.random.default_rng(seed)
    pts = np.meshgrid(*[np.linspace(-0.5 * L[a], 0.5 * L[a], n[a] + 2)[1:-1] for a in range(3)], indexing="ij")
    r2 = sum(p * p for p in pts).reshape(-1)
    return 0.15 * r2 - 0.4 * np.exp(-r2) + 0.01 * rng.normal(size=r2.size)


SPECTRA = {"separated": ((8, 7, 9), (7.0, 6.5, 8.0)), "near_degenerate": ((12, 11, 13), (11.05, 10.2, 11.9))}


@pytest.fixture(scope="module")
def spectra(orc):
    out = {}
    for name, (n, L) in SPECTRA.items():
        og = orc.Grid(n, L)
        v = _well(n, L, 3)
        out[name] = (n, L, v, np.linalg.eigvalsh(_dense_h(og, v))[:16])
    return out


@pytest.mark.parametrize("precision,ptol", [(0, 6), (0, 8), (1, 6)], ids=["fp64-6", "fp64-8", "mixed-6"])
@pytest.mark.parametrize("spectrum,corrflag,maxsub", [("separated", 1, 128), ("separated", 3, 128),
                                                      ("near_degenerate", 1, 128), ("near_degenerate", 1, 40)])
def test_sixteen_roots(pg, torch, spectra, spectrum, corrflag, maxsub, precision, ptol):
    # 16 roots, checked against the dense spectrum.  The reference algorithm
    # does not finish these cases: its restart keeps locked vectors that are
    # orthogonal to the new Ritz vectors only to O(residual / gap), so it locks
    # states twice and lets spurious roots in.  maxsub 40 restarts every two
    # iterations.  Eigenvalue error <= |r|^2 / (gap to level 17), i.e.
    # <= 1e-12 / 0.0068 at ptol 6 (the mixed form ends with an FP64
    # Rayleigh-Ritz step).
    n, L, v, ref = spectra[spectrum]
    grid = pg.Grid(n, L)
    ev, vec, st = grid.solve(dev(torch, v), nroots=16, maxsub=maxsub, maxiter=400, ptol=ptol, corrflag=corrflag,
                             precision=precision, refine=1)
    assert st["nconv"] == 16
    assert np.max(np.abs(ev - ref)) < 1e-8
    V = host(vec)
    assert np.max(np.abs(V @ V.T - np.eye(16))) < 1e-8


def test_kinetic_preconditioner_outside_its_domain_reports_not_converged(pg, torch, spectra):
    # corrflag 3 preconditions with (T - lambda)^-1, which is definite only for
    # states below the lowest kinetic level (bound anions).  In this well the
    # levels lie far inside the kinetic spectrum and the corrections stall: the
    # solve says so instead of returning unconverged values as converged.
    n, L, v, _ = spectra["near_degenerate"]
    grid = pg.Grid(n, L)
    with pytest.raises(pg.NotConverged):
        grid.solve(dev(torch, v), nroots=4, maxsub=40, maxiter=60, ptol=6, corrflag=3)


def test_cluster_without_waters_is_a_box(pg, torch):
    n, L = (24, 20, 28), (20.0, 18.0, 22.0)
    ev, _, _ = pg.cluster_solve(n, L, np.zeros((0, 9)), nroots=2, maxsub=30, ptol=8)
    box = np.array([sum((np.pi * k / (L[a])) ** 2 / 2 for a, k in enumerate(q))
                    for q in [(1, 1, 1), (1, 1, 2), (1, 2, 1), (2, 1, 1)]])
    assert np.max(np.abs(np.asarray(ev) - np.sort(box)[:2])) < 1e-6


def test_argument_limits(pg, torch):
    grid = pg.Grid((8, 8, 8), (6.0, 6.0, 6.0))
    v = torch.zeros(grid.N, dtype=torch.float64, device="cuda")
    for kw in (dict(nroots=0), dict(nroots=17, maxsub=40), dict(nroots=4, maxsub=4), dict(nroots=2, maxsub=129)):
        with pytest.raises(pg.PiscesError) as e:
            grid.solve(v, **kw)
        assert e.value.status == pg.PG_BAD_ARG
    for n in ((1, 8, 8), (8, 1025, 8)):
        with pytest.raises(pg.PiscesError) as e:
            pg.Grid(n, (6.0, 6.0, 6.0))
        assert e.value.status == pg.PG_BAD_ARG
    with pytest.raises(pg.PiscesError) as e:
        pg.Grid((8, 8, 8), (6.0, -1.0, 6.0))
    assert e.value.status == pg.PG_BAD_ARG
    # still serving after the rejected calls
    ev, _, _ = grid.solve(v, nroots=1, ptol=8)
    assert abs(ev[0] - 3 * (np.pi / 6.0) ** 2 / 2) < 1e-9


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("bad", [float("nan"), float("inf")], ids=["nan", "inf"])
def test_nonfinite_product_is_a_numeric_status(pg, torch, precision, bad):
    """A matvec callback that writes one NaN or Inf into Z: the drop-in loop
    must end in PG_NUMERIC, in the FP64 form and in the mixed form (whose
    subspace products read double-float copies of Z), and the handle must
    serve a clean solve afterwards."""
    import ctypes
    n, L = (12, 11, 13), (10.0, 9.0, 11.0)
    grid = pg.Grid(n, L)
    N, nroots, maxsub = grid.N, 2, 16
    rng = np.random.default_rng(4)
    v = dev(torch, -0.5 * np.exp(-0.1 * rng.uniform(0, 30, N)))
    diag = grid.diagonal(v)

    def run(poison_call):
        B = torch.zeros(maxsub * N, dtype=torch.float64, device="cuda")
        Z = torch.zeros_like(B)
        work = torch.zeros(pg.Davidson.work_size(N, maxsub, nroots, 1), dtype=torch.float64, device="cuda")
        B[:N] = grid.piab()
        B[N:2 * N] = dev(torch, np.random.default_rng(3).uniform(-1, 1, N))
        evals = np.zeros(nroots)
        nconv = ctypes.c_int(0)
        inout = np.zeros(3, dtype=np.int32)
        dav = pg.Davidson()
        dav.set_arithmetic(precision)
        ret, calls = 1, 0
        while ret != 0:
            s, ret = dav.step(N, maxsub, nroots, 100, 6, 1, evals, nconv, B, Z, diag, work, inout)
            if s != pg.PG_OK:
                return s, calls
            if ret == 1:
                i0, z0, k = (int(a) for a in inout)
                grid.hx(v, B[i0 * N:(i0 + k) * N], nvec=k, out=Z[z0 * N:(z0 + k) * N], precision=precision)
                if calls == poison_call:
                    Z[z0 * N + N // 3] = bad
                calls += 1
        return pg.PG_OK, calls

    s, calls = run(poison_call=2)
    assert s == pg.PG_NUMERIC and calls == 3, (s, calls)
    s, calls = run(poison_call=-1)
    assert s == pg.PG_OK and calls > 3
