"""The kinetic preconditioner R <- (T - sigma_j)^-1 R (pg_kinetic_precondition):
the FP16-split tensor-core kernel of the mixed form (k_kin_f16: xy forward
transforms of the planes, z forward transform + diagonal + z backward
transform of 128-line tiles, xy backward transforms, one persistent launch)
against the FP64 axis passes and against a numpy restatement of the
operator; the split-TF32 axis passes it replaces; shifts at the denominator
floor; blocks scaled by 1e-20 and 1e20; more vectors than one launch takes;
the periodic FFT kinetic term (a non-symmetric eigenbasis); bit for bit run
to run and on two streams; a NaN stays in its own vector; grids the kernel
declines fall back to the axis passes; a solve gives the same eigenpairs
with either mixed preconditioner.

Tolerance: 2e-5 of max |M R| (the mixed form's H*X bound: FP16 or TF32 high
and low parts, three products, FP32 accumulation, and the diagonal in
FP32)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-5


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def rand_block(torch, grid, k, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn(k * grid.N, dtype=torch.float64, device="cuda", generator=g)


def rel_err(a, b):
    return float((a - b).abs().max()) / float(b.abs().max())


def apply(grid, R, sigma, precision, pg):
    Y = R.clone()
    grid.precondition(Y, sigma, precision=precision)
    return Y


def numpy_precondition(n, L, R, sigma):
    """(T - sigma)^-1 R on a cubic sine-DVR grid in FP64: the DST-I eigenbasis
    Q[i][k] = sqrt(2/(n+1)) sin(pi (i+1)(k+1)/(n+1)), d_k = (pi (k+1)/L)^2/2,
    |denominator| at least a tenth of the lowest level."""
    i = np.arange(n)
    Q = np.sqrt(2.0 / (n + 1)) * np.sin(np.pi * np.outer(i + 1, i + 1) / (n + 1))
    d = 0.5 * (np.pi * (i + 1) / L) ** 2
    floor = 0.1 * 3 * 0.5 * (np.pi / L) ** 2
    out = []
    for r, s in zip(R.reshape(len(sigma), n, n, n), sigma):  # [z][y][x]
        c = np.einsum("kz,jy,ix,zyx->kji", Q, Q, Q, r)
        den = d[:, None, None] + d[None, :, None] + d[None, None, :] - s
        den = np.where(np.abs(den) < floor, np.where(den < 0, -floor, floor), den)
        out.append(np.einsum("kz,jy,ix,zyx->kji", Q, Q, Q, c / den))
    return np.stack(out).reshape(-1)


@pytest.mark.parametrize("n,k", [(16, 3), (32, 5), (48, 4), (64, 4), (80, 2), (96, 8)])
def test_kin_f16_matches_fp64_and_tf32(pg, torch, n, k):
    L = 0.625 * (n + 1)
    grid = pg.Grid(n, L)
    assert "k_kin_f16" in grid.precond_plan()
    R = rand_block(torch, grid, k, n)
    # shifts below the kinetic spectrum (Ritz values of bound states), and
    # just below and just above its lowest level, where |T - sigma| meets the
    # floor (a tenth of that level).  The diagonal is FP32 in the mixed form:
    # shifts within ~1e-7 of a level, where FP32 and FP64 may round the
    # denominator to opposite signs, are avoided.
    lo = 3 * 0.5 * (np.pi / L) ** 2
    sigma = np.array([-0.05, lo - 0.3, 0.97 * lo, 1.03 * lo, -0.5, 0.5 * lo, -1.0, -0.001][:k])
    y64 = apply(grid, R, sigma, pg.PG_FP64, pg)
    y16 = apply(grid, R, sigma, pg.PG_MIXED, pg)
    assert rel_err(y16, y64) <= TOL
    for j in range(k):  # every vector, not only the largest
        a, b = y16[j * grid.N:(j + 1) * grid.N], y64[j * grid.N:(j + 1) * grid.N]
        assert rel_err(a, b) <= TOL, j
    grid.set_precond_kernel(1)
    assert "axis passes" in grid.precond_plan()
    ytf = apply(grid, R, sigma, pg.PG_MIXED, pg)
    assert rel_err(ytf, y64) <= TOL
    if n <= 32:
        ref = numpy_precondition(n, L, R.cpu().numpy(), sigma)
        assert float(np.abs(y64.cpu().numpy() - ref).max()) <= 1e-12 * float(np.abs(ref).max())


@pytest.mark.parametrize("scale", [1e-20, 1e20])
def test_kin_f16_scaled_blocks(pg, torch, scale):
    grid = pg.Grid(48, 30.0)
    R = rand_block(torch, grid, 3, 7) * scale
    sigma = [-0.02, -0.01, 0.005]
    assert rel_err(apply(grid, R, sigma, pg.PG_MIXED, pg), apply(grid, R, sigma, pg.PG_FP64, pg)) <= TOL


def test_kin_f16_more_vectors_than_one_launch(pg, torch):
    grid = pg.Grid(16, 10.0)
    R = rand_block(torch, grid, 40, 11)
    sigma = np.linspace(-0.5, 0.1, 40)
    assert rel_err(apply(grid, R, sigma, pg.PG_MIXED, pg), apply(grid, R, sigma, pg.PG_FP64, pg)) <= TOL


def test_kin_f16_fft_grid(pg, torch):
    # periodic FFT kinetic term: the real Fourier basis is not symmetric, so
    # the forward and backward images differ
    grid = pg.Grid(32, 20.0, dvrtype=3)
    assert "k_kin_f16" in grid.precond_plan()
    R = rand_block(torch, grid, 4, 5)
    sigma = [-0.1, 0.0, 0.025, -0.5]  # 0.0: the constant mode meets the floor
    assert rel_err(apply(grid, R, sigma, pg.PG_MIXED, pg), apply(grid, R, sigma, pg.PG_FP64, pg)) <= TOL


def test_kin_f16_repeats_and_two_streams(pg, torch):
    grid = pg.Grid(64, 40.0)
    R1 = rand_block(torch, grid, 4, 3)
    R2 = rand_block(torch, grid, 4, 4)
    sigma = [-0.02, -0.015, -0.01, -0.005]
    ref1 = apply(grid, R1, sigma, pg.PG_MIXED, pg)
    ref2 = apply(grid, R2, sigma, pg.PG_MIXED, pg)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    outs = []
    for _ in range(3):
        a, b = R1.clone(), R2.clone()
        torch.cuda.synchronize()
        grid.precondition(a, sigma, stream=s1.cuda_stream)
        grid.precondition(b, sigma, stream=s2.cuda_stream)
        outs.append((a, b))
    torch.cuda.synchronize()
    for a, b in outs:
        assert torch.equal(a, ref1) and torch.equal(b, ref2)


def test_kin_f16_nan_stays_in_its_vector(pg, torch):
    grid = pg.Grid(32, 20.0)
    R = rand_block(torch, grid, 3, 9)
    R[5] = float("nan")
    sigma = [-0.1, -0.05, 0.0]
    y = apply(grid, R, sigma, pg.PG_MIXED, pg)
    N = grid.N
    assert bool(torch.isnan(y[:N]).any())
    y64 = apply(grid, R, sigma, pg.PG_FP64, pg)
    assert rel_err(y[N:], y64[N:]) <= TOL


@pytest.mark.parametrize("shape,why", [((33, 33, 33), "odd nx"), ((48, 48, 40), "differ"),
                                       ((112, 112, 112), "more than 96")])
def test_kin_f16_declines(pg, torch, shape, why):
    grid = pg.Grid(shape, 30.0)
    plan = grid.precond_plan()
    assert "axis passes" in plan and why in plan
    R = rand_block(torch, grid, 2, 1)
    sigma = [-0.05, 0.02]
    assert rel_err(apply(grid, R, sigma, pg.PG_MIXED, pg), apply(grid, R, sigma, pg.PG_FP64, pg)) <= TOL


def test_solve_with_either_mixed_preconditioner(pg, torch, clusters):
    # (H2O)12 on 48^3: the mixed solve with the FP16 preconditioner and with
    # the TF32 axis passes reach the same eigenpairs
    w = clusters.water_cluster(12, 7.0, 5)
    grid = pg.Grid(48, 30.0)
    v = grid.potential(pg.WaterTables(w))
    res = []
    for kind in (0, 1):
        grid.set_precond_kernel(kind)
        ev, vec, st = grid.solve(v, nroots=2, maxsub=24, maxiter=200, ptol=6, corrflag=3, precision=pg.PG_MIXED)
        res.append((ev, vec, st))
    (e0, v0, s0), (e1, v1, s1) = res
    assert np.abs(np.asarray(e0) - np.asarray(e1)).max() <= 1e-10
    assert abs(s0["n_matvec"] - s1["n_matvec"]) <= 4
    ov = torch.abs(torch.sum(v0 * v1, dim=1)) / (v0.norm(dim=1) * v1.norm(dim=1))
    assert float(ov.min()) >= 1 - 1e-8, ov
