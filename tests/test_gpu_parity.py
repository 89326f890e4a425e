"""GPU parity: the CUDA path through the C ABI against the golden vectors of
the reference CPU code and against the CPU oracle on the same inputs.

Tolerances: V(r) and diag(H) 1e-13 relative to max|V| (the kernel evaluates
the reference's expressions in its order without fused multiply-adds; exp
may differ in the last place); FP64 H*X 1e-13 relative to max|Y|;
eigenvalues of the FP64 path 1e-8 Eh of the reference, eigenvector overlap
>= 1 - 1e-8.
"""
import numpy as np
import pytest

from conftest import golden, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def dev(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def host(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("tag", ["w6", "w24"])
def test_potential_from_reference_tables(pg, torch, tag):
    g = golden(f"dpp_{tag}.npz")
    grid = pg.Grid(g["n"], g["L"])
    t = pg.WaterTables.from_lists(g["sites"], g["charges"], g["charge_site"], g["dipoles"], g["dipole_site"])
    v, parts = grid.potential(t, parts=True)
    scale = np.max(np.abs(g["v"]))
    assert np.max(np.abs(host(v) - g["v"])) / scale < 1e-13
    for k, name in enumerate(["v_pc", "v_ind", "v_rep", "v_pol"]):
        assert np.max(np.abs(host(parts[k]) - g[name])) / scale < 1e-13, name
    assert rel(host(grid.diagonal(v)), g["diag"]) < 1e-13


@pytest.mark.parametrize("tag", ["w6", "w24"])
def test_potential_from_own_site_producer(pg, torch, tag):
    g = golden(f"dpp_{tag}.npz")
    grid = pg.Grid(g["n"], g["L"])
    v = grid.potential(pg.WaterTables(g["waters"]))
    assert rel(host(v), g["v"]) < 1e-12


def test_potential_ions(pg, torch):
    g = golden("ions_small.npz")
    grid = pg.Grid(g["n"], g["L"])
    v = grid.potential(pg.WaterTables(g["waters"]))
    grid.add_ions(v, g["ion_sites"], g["ion_charges"])
    assert rel(host(v), g["v"]) < 1e-12


def test_potential_point_on_a_site(pg, orc, torch):
    # a grid point exactly on a site exercises the damped branches (R < r0)
    # and the R = 0 limits of every term (src/Potential.cpp:1191, 1252, 1357)
    g = golden("dpp_w6.npz")
    n, L = (9, 9, 9), (10.0, 10.0, 10.0)
    ogrid = orc.Grid(n, L)
    sites = np.array(g["sites"], dtype=np.float64)
    sites[0:3] = [ogrid.x[0][4], ogrid.x[1][4], ogrid.x[2][4]]      # O of water 0 on the centre point
    sites[12 + 9:12 + 12] = [ogrid.x[0][2], ogrid.x[1][6], ogrid.x[2][3]]  # M of water 1 on a grid point
    ref = ogrid.potential_dpp(sites, g["charges"], g["charge_site"], g["dipoles"], g["dipole_site"])
    assert np.all(np.isfinite(ref))
    grid = pg.Grid(n, L)
    t = pg.WaterTables.from_lists(sites, g["charges"], g["charge_site"], g["dipoles"], g["dipole_site"])
    assert rel(host(grid.potential(t)), ref) < 1e-13


def test_spherical_potential(pg, orc, torch):
    n, L = (11, 12, 13), (12.0, 13.0, 14.0)
    assert rel(host(pg.Grid(n, L).spherical(0.1)), orc.Grid(n, L).spherical(0.1)) < 1e-15


@pytest.mark.parametrize("name", ["dpp_w6.npz", "dpp_w24.npz", "small_w6.npz", "ions_small.npz"])
def test_hx_fp64_matches_reference(pg, torch, name):
    g = golden(name)
    grid = pg.Grid(g["n"], g["L"])
    y = grid.hx(dev(torch, g["v"]), dev(torch, g["mv_x"]))
    assert rel(host(y), g["mv_y"]) < 1e-13


def test_hx_fp64_block_matches_oracle(pg, orc, torch):
    # 7 vectors: exercises the 4-vector register groups and a ragged tail
    n, L = (24, 20, 28), (20.0, 18.0, 22.0)
    rng = np.random.default_rng(5)
    v = rng.normal(size=int(np.prod(n)))
    X = rng.normal(size=(7, int(np.prod(n))))
    grid = pg.Grid(n, L)
    Y = host(grid.hx(dev(torch, v), dev(torch, X))).reshape(7, -1)
    og = orc.Grid(n, L)
    for r in range(7):
        assert rel(Y[r], og.matvec(v, X[r])) < 1e-13


def test_hx_fp64_properties_at_64cubed(pg, orc, torch):
    # full C2 grid: symmetry <x, H y> = <H x, y>, linearity, and one vector vs the oracle
    g = golden("dpp_w24.npz")
    n, L = (64, 64, 64), (40.0, 40.0, 40.0)
    grid = pg.Grid(n, L)
    v = grid.potential(pg.WaterTables(g["waters"]))
    rng = np.random.default_rng(11)
    X = dev(torch, rng.normal(size=(2, grid.N)))
    Y = grid.hx(v, X).view(2, -1)
    a = float((X[0] * Y[1]).sum())
    b = float((Y[0] * X[1]).sum())
    assert abs(a - b) < 1e-11 * (abs(a) + abs(b))
    Z = grid.hx(v, (2.0 * X[0] - 3.0 * X[1]).contiguous())
    assert float((Z - (2.0 * Y[0] - 3.0 * Y[1])).abs().max()) < 1e-11 * float(Y.abs().max())
    og = orc.Grid(n, L)
    assert rel(host(Y[0]), og.matvec(host(v), host(X[0]))) < 1e-13


def test_solve_fp64_two_states(pg, torch):
    g = golden("small_w6.npz")
    grid = pg.Grid(g["n"], g["L"])
    ev, vec, st = grid.solve(dev(torch, g["v"]), nroots=2, ptol=8)
    assert st["nconv"] == 2
    assert np.max(np.abs(ev - g["evals"])) < 1e-8
    W = g["wavefn"].reshape(2, -1)
    V = host(vec)
    for r in range(2):
        assert abs(V[r] @ W[r]) / np.linalg.norm(V[r]) / np.linalg.norm(W[r]) > 1 - 1e-8


def test_solve_fp64_c1(pg, torch):
    # (H2O)6, 32^3 over 30 bohr, lowest state, from water coordinates
    g = golden("c1.npz")
    ev, vec, st = pg.cluster_solve(g["n"], g["L"], g["waters"], nroots=1, ptol=8)
    assert abs(ev[0] - g["evals"][0]) < 1e-8
    w = g["wavefn32"].astype(np.float64)
    assert abs(vec[0] @ w) / np.linalg.norm(vec[0]) / np.linalg.norm(w) > 1 - 1e-8


def test_solve_fp64_matches_oracle_iteration_count(pg, orc, torch):
    # same start vectors, same algorithm: the matvec counts agree closely
    g = golden("small_w6.npz")
    grid = pg.Grid(g["n"], g["L"])
    ev, vec, st = grid.solve(dev(torch, g["v"]), nroots=2, ptol=8)
    _, ev_o, _, nmv_o = orc.Grid(g["n"], g["L"]).solve(g["v"], nstates=2, ptol=8)
    assert np.max(np.abs(ev - ev_o)) < 1e-10
    assert abs(st["n_matvec"] - nmv_o) <= max(8, nmv_o // 20)


@pytest.mark.parametrize("corrflag", [0, 2], ids=["residual", "jacobi-davidson"])
def test_solve_fp64_other_corrections_match_oracle(pg, orc, torch, corrflag):
    # the reference's other DiagMethods: 4/5 -> corrflag 0 (plain residual),
    # 3 -> corrflag 2 (zeroth-order Jacobi-Davidson, src/Davidson.cpp:530-549)
    g = golden("small_w6.npz")
    grid = pg.Grid(g["n"], g["L"])
    ev, vec, st = grid.solve(dev(torch, g["v"]), nroots=2, ptol=8, corrflag=corrflag)
    sto, ev_o, _, nmv_o = orc.Grid(g["n"], g["L"]).solve(g["v"], nstates=2, ptol=8, corrflag=corrflag)
    assert sto == 2 and st["nconv"] == 2
    assert np.max(np.abs(ev - ev_o)) < 1e-10
    assert np.max(np.abs(ev - g["evals"][:2])) < 1e-8
    assert abs(st["n_matvec"] - nmv_o) <= max(8, nmv_o // 20)


def test_solve_analytic(pg, torch):
    g = golden("analytic.npz")
    grid = pg.Grid(g["box_n"], g["box_L"])
    v0 = torch.zeros(grid.N, dtype=torch.float64, device="cuda")
    ev, _, _ = grid.solve(v0, nroots=1, ptol=8)
    assert abs(ev[0] - sum((3.14159265358979 / L) ** 2 / 2 for L in g["box_L"])) < 1e-9
    grid = pg.Grid(g["harm_n"], g["harm_L"])
    ev, _, _ = grid.solve(grid.spherical(float(g["harm_k"])), nroots=1, ptol=8)
    assert abs(ev[0] - g["harm_evals"][0]) < 1e-9
    grid = pg.Grid(g["full_n"], g["full_L"])
    ev, _, _ = grid.solve(dev(torch, g["full_v"]), nroots=3, ptol=8, maxsub=40)
    assert np.max(np.abs(ev - g["full_evals"][:3])) < 1e-9


def test_solve_not_converged_is_a_status(pg, torch):
    g = golden("small_w6.npz")
    grid = pg.Grid(g["n"], g["L"])
    with pytest.raises(pg.NotConverged):
        grid.solve(dev(torch, g["v"]), nroots=2, ptol=8, maxiter=1)


def test_reverse_communication_drop_in(pg, torch):
    # Drive pg_davidson_rci exactly as DVR::davdriver drives Davidson()
    # (src/davdriver.cpp:58-86), with pg_hx as the matvec callback.
    import ctypes
    g = golden("small_w6.npz")
    grid = pg.Grid(g["n"], g["L"])
    N, nroots, maxsub = grid.N, 2, 20
    v = dev(torch, g["v"])
    B = torch.zeros(maxsub * N, dtype=torch.float64, device="cuda")
    Z = torch.zeros_like(B)
    work = torch.zeros(pg.Davidson.work_size(N, maxsub, nroots, 1), dtype=torch.float64, device="cuda")
    diag = grid.diagonal(v)
    B[:N] = grid.piab()
    B[N:2 * N] = dev(torch, np.random.default_rng(3).uniform(-1, 1, N))
    evals = np.zeros(nroots)
    nconv = ctypes.c_int(0)
    inout = np.zeros(3, dtype=np.int32)
    dav = pg.Davidson()
    ret, calls = 1, 0
    while ret != 0:
        s, ret = dav.step(N, maxsub, nroots, 100, 8, 1, evals, nconv, B, Z, diag, work, inout)
        assert s == pg.PG_OK
        if ret == 1:
            i0, z0, k = (int(a) for a in inout)
            grid.hx(v, B[i0 * N:(i0 + k) * N], nvec=k, out=Z[z0 * N:(z0 + k) * N])
            calls += 1
    assert nconv.value == 2 and calls > 5
    assert np.max(np.abs(evals - g["evals"])) < 1e-8


def test_reverse_communication_mixed_arithmetic(pg, torch):
    # the same drop-in loop with the mixed form: double-float subspace
    # arithmetic on the handle (its twins of the caller's B and Z), mixed H*X
    # in the callback; residual 1e-6, eigenvalues within 1e-6 Eh.  The
    # arithmetic cannot change while the solve is in progress.
    import ctypes
    g = golden("small_w6.npz")
    grid = pg.Grid(g["n"], g["L"])
    N, nroots, maxsub = grid.N, 2, 20
    v = dev(torch, g["v"])
    B = torch.zeros(maxsub * N, dtype=torch.float64, device="cuda")
    Z = torch.zeros_like(B)
    work = torch.zeros(pg.Davidson.work_size(N, maxsub, nroots, 1), dtype=torch.float64, device="cuda")
    diag = grid.diagonal(v)
    B[:N] = grid.piab()
    B[N:2 * N] = dev(torch, np.random.default_rng(3).uniform(-1, 1, N))
    evals = np.zeros(nroots)
    nconv = ctypes.c_int(0)
    inout = np.zeros(3, dtype=np.int32)
    dav = pg.Davidson()
    dav.set_arithmetic(pg.PG_MIXED)
    ret, calls = 1, 0
    while ret != 0:
        s, ret = dav.step(N, maxsub, nroots, 100, 6, 1, evals, nconv, B, Z, diag, work, inout)
        assert s == pg.PG_OK
        if calls == 1:
            with pytest.raises(pg.PiscesError) as e:
                dav.set_arithmetic(pg.PG_FP64)
            assert e.value.status == pg.PG_BAD_ARG
        if ret == 1:
            i0, z0, k = (int(a) for a in inout)
            grid.hx(v, B[i0 * N:(i0 + k) * N], nvec=k, out=Z[z0 * N:(z0 + k) * N], precision=pg.PG_MIXED)
            calls += 1
    assert nconv.value == 2 and calls > 5
    assert np.max(np.abs(evals - g["evals"])) < 1e-6
    # the handle is free again once the solve has ended
    dav.set_arithmetic(pg.PG_FP64)


# ---------------------------------------------------------------- mixed form
# split-TF32 tensor-core kinetic contractions, FP32 accumulation: each output
# carries an absolute error of about 2^-21 * sum_b |T_ib x_b|, so the bound is
# stated against max|Y| of the FP64 product.
MIXED_HX_TOL = 2e-5


@pytest.mark.parametrize("n,L,nvec", [((24, 20, 28), (20.0, 18.0, 22.0), 7), ((64, 64, 64), (40.0, 40.0, 40.0), 4),
                                      ((33, 48, 17), (30.0, 40.0, 16.0), 3), ((96, 96, 96), (48.0, 48.0, 48.0), 1)])
def test_hx_mixed_matches_fp64(pg, torch, n, L, nvec):
    grid = pg.Grid(n, L)
    rng = np.random.default_rng(7)
    v = dev(torch, rng.normal(size=grid.N))
    X = dev(torch, rng.normal(size=nvec * grid.N))
    y64 = host(grid.hx(v, X, precision=pg.PG_FP64))
    ymx = host(grid.hx(v, X, precision=pg.PG_MIXED))
    assert np.max(np.abs(ymx - y64)) / np.max(np.abs(y64)) < MIXED_HX_TOL


def test_hx_mixed_smooth_vector(pg, torch):
    # an eigenfunction-like input: the kinetic sums cancel strongly
    g = golden("small_w6.npz")
    grid = pg.Grid(g["n"], g["L"])
    v = dev(torch, g["v"])
    W = dev(torch, g["wavefn"])
    y64 = host(grid.hx(v, W, precision=pg.PG_FP64))
    ymx = host(grid.hx(v, W, precision=pg.PG_MIXED))
    # H psi ~ E psi is small while the kinetic terms are not: bound the error
    # by the size of the terms, sum over axes of max row sum |T| times max|x|
    scale = sum(np.abs(grid.kinetic(a)).sum(axis=1).max() for a in range(3)) * np.abs(g["wavefn"]).max()
    assert np.max(np.abs(ymx - y64)) / scale < 2e-6
    # Rayleigh quotients agree far better than the pointwise bound
    Wh = g["wavefn"].reshape(2, -1)
    for r in range(2):
        a = Wh[r] @ y64.reshape(2, -1)[r] / (Wh[r] @ Wh[r])
        b = Wh[r] @ ymx.reshape(2, -1)[r] / (Wh[r] @ Wh[r])
        assert abs(a - b) < 1e-7


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solve_kinetic_preconditioner(pg, torch, precision):
    # corrflag 3 (exact kinetic preconditioner) converges to the same
    # eigenpairs as the reference algorithm, in far fewer products
    g = golden("small_w6.npz")
    grid = pg.Grid(g["n"], g["L"])
    prec = pg.PG_FP64 if precision == "fp64" else pg.PG_MIXED
    ptol = 8 if precision == "fp64" else 6
    ev3, vec3, st3 = grid.solve(dev(torch, g["v"]), nroots=2, ptol=ptol, corrflag=3, precision=prec)
    ev1, _, st1 = grid.solve(dev(torch, g["v"]), nroots=2, ptol=ptol, corrflag=1, precision=prec)
    assert np.max(np.abs(ev3 - g["evals"])) < (1e-8 if precision == "fp64" else 1e-6)
    assert st3["n_matvec"] < st1["n_matvec"]
    W = g["wavefn"].reshape(2, -1)
    V = host(vec3)
    for r in range(2):
        assert abs(V[r] @ W[r]) / np.linalg.norm(V[r]) / np.linalg.norm(W[r]) > 1 - 1e-8


def test_solve_kinetic_preconditioner_c1(pg, torch):
    g = golden("c1.npz")
    ev, vec, st = pg.cluster_solve(g["n"], g["L"], g["waters"], nroots=1, ptol=8, corrflag=3)
    assert abs(ev[0] - g["evals"][0]) < 1e-8
    w = g["wavefn32"].astype(np.float64)
    assert abs(vec[0] @ w) / np.linalg.norm(vec[0]) / np.linalg.norm(w) > 1 - 1e-8


def test_solve_mixed_c1_within_1e6(pg, torch):
    g = golden("c1.npz")
    ev, vec, st = pg.cluster_solve(g["n"], g["L"], g["waters"], nroots=1, ptol=6, precision=pg.PG_MIXED, refine=1)
    assert abs(ev[0] - g["evals"][0]) < 1e-6
    w = g["wavefn32"].astype(np.float64)
    assert abs(vec[0] @ w) / np.linalg.norm(vec[0]) / np.linalg.norm(w) > 1 - 1e-8


# ---------------------------------------------------------------- block products

@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("n,na,nb", [(64 ** 3, 40, 4), (33 ** 3, 5, 5), (1000, 1, 128), (4097, 16, 16)])
def test_block_gram(pg, torch, precision, n, na, nb):
    """S = P Q^T against torch FP64; the double-float form within 1e-12 of
    the largest |entry| scale (|P_a| |Q_b|)."""
    g = torch.Generator(device="cuda").manual_seed(11)
    P = torch.randn(na, n, dtype=torch.float64, device="cuda", generator=g)
    Q = torch.randn(nb, n, dtype=torch.float64, device="cuda", generator=g)
    ref = P @ Q.T
    out = pg.block_gram(P, Q, precision=precision)
    torch.cuda.synchronize()
    scale = float(P.norm(dim=1).max() * Q.norm(dim=1).max())
    err = float((out - ref).abs().max()) / scale
    assert err <= (1e-14 if precision == 0 else 1e-12), err
    again = pg.block_gram(P, Q, precision=precision)
    assert torch.equal(out, again)  # deterministic


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("n,na,ny", [(64 ** 3, 40, 4), (33 ** 3, 7, 16), (999, 128, 1)])
def test_block_combine(pg, torch, precision, n, na, ny):
    g = torch.Generator(device="cuda").manual_seed(12)
    P = torch.randn(na, n, dtype=torch.float64, device="cuda", generator=g)
    Cm = torch.randn(na, ny, dtype=torch.float64, device="cuda", generator=g)
    ref = Cm.T @ P
    out = pg.block_combine(P, Cm, precision=precision)
    torch.cuda.synchronize()
    scale = float(Cm.abs().sum(dim=0).max()) * float(P.abs().max())
    err = float((out - ref).abs().max()) / scale
    assert err <= (1e-14 if precision == 0 else 1e-12), err


@pytest.mark.gpu
@pytest.mark.parametrize("n,na,nq", [(262144, 40, 4), (1000, 7, 3), (4097, 16, 16)])
def test_block_products_on_twins(pg, torch, n, na, nq):
    # the twin-input forms the mixed Davidson launches: the same products as
    # the FP64-input mixed entry points (which split their inputs on the fly)
    g = torch.Generator(device="cuda").manual_seed(n + na)
    P = torch.randn(na, n, dtype=torch.float64, device="cuda", generator=g)
    Q = torch.randn(nq, n, dtype=torch.float64, device="cuda", generator=g)
    Cm = torch.randn(na, nq, dtype=torch.float64, device="cuda", generator=g)
    Pt, Qt = pg.split_twin(P), pg.split_twin(Q)
    hi_lo = Pt.view(torch.float32).view(na, n, 2).double()
    assert float((hi_lo.sum(-1) - P).abs().max()) <= 2.0 ** -46 * float(P.abs().max())
    S = pg.block_gram_twin(Pt, Qt)
    torch.cuda.synchronize()
    ref = P @ Q.T
    scale = float(P.abs().max()) * float(Q.abs().max()) * n
    assert float((S - ref).abs().max()) / scale <= 1e-14
    assert float((S - pg.block_gram(P, Q, precision=pg.PG_MIXED)).abs().max()) / scale <= 1e-15
    Yt = torch.empty(nq, n, dtype=torch.float64, device="cuda")
    Y = pg.block_combine_twin(Pt, Cm, out_twin=Yt)
    torch.cuda.synchronize()
    cscale = float(Cm.abs().sum(dim=0).max()) * float(P.abs().max())
    assert float((Y - Cm.T @ P).abs().max()) / cscale <= 1e-12
    # the twin written beside Y is the accumulator pair: hi + lo = Y to 2^-46
    yhl = Yt.view(torch.float32).view(nq, n, 2).double().sum(-1)
    assert float((yhl - Y).abs().max()) <= 2.0 ** -46 * float(Y.abs().max())


# ---------------------------------------------------------------- c2 workload

def _c2(pg, torch):
    gd = golden("c2.npz")
    grid = pg.Grid(tuple(int(x) for x in gd["n"]), tuple(float(x) for x in gd["L"]))
    v = grid.potential(pg.WaterTables(gd["waters"]))
    return gd, grid, v


@pytest.mark.gpu
def test_solve_c2_reference_algorithm(pg, torch):
    """(H2O)24, 64^3, 4 states, maxsub 60, residual 1e-8, the reference's
    diagonal correction: eigenvalues within 1e-8 Eh of the reference run and
    the same number of H*x products as the oracle's restatement of the
    reference algorithm needs on this input (4500)."""
    gd, grid, v = _c2(pg, torch)
    ev, vec, st = grid.solve(v, nroots=4, maxsub=60, maxiter=400, ptol=8, corrflag=1)
    assert np.max(np.abs(np.asarray(ev) - gd["evals"])) <= 1e-8
    assert st["n_matvec"] == 4500


@pytest.mark.gpu
def test_solve_c2_mixed_against_fp64_and_reference(pg, torch):
    """The mixed form (split-TF32 H*X, double-float subspace, FP64 refinement)
    against the FP64 form with the same corrections: |dE| <= 1e-6 Eh per
    eigenvalue and eigenvector overlap >= 1 - 1e-8; both against the reference
    eigenvalues, and the FP64 vectors against the reference's (stored in
    float16, so overlap >= 1 - 1e-3)."""
    gd, grid, v = _c2(pg, torch)
    e64, x64, _ = grid.solve(v, nroots=4, maxsub=60, maxiter=400, ptol=8, corrflag=3)
    emx, xmx, _ = grid.solve(v, nroots=4, maxsub=60, maxiter=400, ptol=6, corrflag=3, precision=pg.PG_MIXED,
                             refine=1)
    e64, emx = np.asarray(e64), np.asarray(emx)
    assert np.max(np.abs(e64 - gd["evals"])) <= 1e-8
    assert np.max(np.abs(emx - e64)) <= 1e-6
    X64 = x64.reshape(4, -1).double()
    XMX = xmx.reshape(4, -1).double()
    ov = torch.abs(torch.sum(X64 * XMX, dim=1)) / (X64.norm(dim=1) * XMX.norm(dim=1))
    assert float(ov.min()) >= 1 - 1e-8, ov
    ref = torch.tensor(gd["wavefn16"].astype(np.float64), device="cuda").reshape(4, -1)
    ov = torch.abs(torch.sum(X64 * ref, dim=1)) / (X64.norm(dim=1) * ref.norm(dim=1))
    assert float(ov.min()) >= 1 - 1e-3, ov


# ---------------------------------------------------------------- FFT kinetic path (DVRType 3)

@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("n,L,nvec", [(24, 20.0, 1), (32, 30.0, 4)])
def test_hx_fft_grid_matches_reference_fft_apply(pg, orc, torch, precision, n, L, nvec):
    """H*X on a DVRType 3 grid against the numpy restatement of
    VectorFFT::apply (cubic grids): FP64 to round-off, mixed within the
    mixed form's H*X bound (2e-5 of max |Y|, as for the sine DVR)."""
    rng = np.random.Generator(np.random.PCG64(4))
    grid = pg.Grid((n, n, n), (L, L, L), dvrtype=3)
    N = grid.N
    x = rng.standard_normal(nvec * N)
    v = rng.standard_normal(N)
    ke = orc.fft_ke_diag((n, n, n), (L, L, L))
    ref = np.concatenate([orc.fft_apply(x[k * N:(k + 1) * N], v, (n, n, n), ke) for k in range(nvec)])
    y = grid.hx(dev(torch, v), dev(torch, x), nvec=nvec, precision=precision)
    err = np.max(np.abs(host(y) - ref)) / np.max(np.abs(ref))
    assert err <= (1e-13 if precision == 0 else 2e-5), err


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_fft_grid_plane_waves_are_eigenvectors(pg, torch, precision):
    """V = 0 on a periodic grid: H applied to a product of axis plane waves
    cos(2 pi m_a i_a / n_a) returns it times sum_a ekin_a[m_a] (known answer
    of the FFT kinetic operator), for a non-cubic box; the ground state of
    the empty box is the constant vector with energy 0."""
    n3, L3 = (16, 12, 20), (15.0, 13.0, 17.0)
    grid = pg.Grid(n3, L3, dvrtype=3)
    ek = [pg.fft_kinetic(n3[a], L3[a])[1] for a in range(3)]
    v = torch.zeros(grid.N, dtype=torch.float64, device="cuda")
    for m in ((0, 0, 0), (1, 0, 0), (3, 2, 1), (8, 6, 10), (5, 11, 7)):
        f = [np.cos(2 * np.pi * m[a] * np.arange(n3[a]) / n3[a]) for a in range(3)]
        x = (f[2][:, None, None] * f[1][None, :, None] * f[0][None, None, :]).reshape(-1)
        e = ek[0][m[0]] + ek[1][m[1]] + ek[2][m[2]]
        y = host(grid.hx(v, dev(torch, x), nvec=1, precision=precision))
        err = np.max(np.abs(y - e * x)) / sum(float(np.max(k)) for k in ek)  # relative to the kinetic scale
        assert err <= (1e-12 if precision == 0 else 2e-5), (m, err)
    for corr in (1, 3):
        ev, _, _ = grid.solve(v, nroots=1, maxsub=20, maxiter=200, ptol=8, corrflag=corr)
        assert abs(ev[0]) <= 1e-8, corr
    # and the sine DVR on the same non-cubic box: the particle-in-a-box ground state
    sine = pg.Grid(n3, L3)
    e0 = sum(0.5 * (np.pi / L) ** 2 for L in L3)
    for corr in (1, 3):
        ev, _, _ = sine.solve(v, nroots=1, maxsub=20, maxiter=200, ptol=8, corrflag=corr)
        assert abs(ev[0] - e0) <= 1e-8, (corr, ev, e0)


@pytest.mark.gpu
def test_fft_grid_cluster_solve_against_dense_reference_operator(pg, orc, torch, clusters):
    """(H2O)4 on a periodic 12^3 grid: the two lowest eigenvalues of the device
    Davidson (FP64, diagonal correction and kinetic preconditioner; mixed)
    against numpy's dense eigensolver of the reference FFT operator, built
    column by column with the restatement of VectorFFT::apply."""
    n, L = 12, 14.0
    w = clusters.water_cluster(4, 4.0, seed=5)
    grid = pg.Grid((n, n, n), (L, L, L), dvrtype=3)
    v = grid.potential(pg.WaterTables(w))
    vh = host(v)
    ke = orc.fft_ke_diag((n, n, n), (L, L, L))
    N = grid.N
    H = np.empty((N, N))
    eye = np.zeros(N)
    for c in range(N):
        eye[c] = 1.0
        H[:, c] = orc.fft_apply(eye, vh, (n, n, n), ke)
        eye[c] = 0.0
    ref = np.linalg.eigvalsh(0.5 * (H + H.T))[:2]
    for corr in (1, 3):
        ev, _, _ = grid.solve(v, nroots=2, maxsub=30, maxiter=300, ptol=8, corrflag=corr)
        assert np.max(np.abs(np.asarray(ev) - ref)) <= 1e-8, (corr, ev, ref)
    ev, _, _ = grid.solve(v, nroots=2, maxsub=30, maxiter=300, ptol=6, corrflag=3, precision=pg.PG_MIXED, refine=1)
    assert np.max(np.abs(np.asarray(ev) - ref)) <= 1e-6


# ---------------------------------------------------------------- waters + ions (c3 model)

@pytest.mark.gpu
def test_solve_waters_and_ions_match_reference(pg, torch):
    """(H2O)8 + Na+ + Cl- on a non-cubic 14 x 16 x 18 grid: V = DPP(waters) +
    Bloomfield(ions), two states, against the reference run of the same
    combined model (ions_small fixture): eigenvalues within 1e-8 Eh."""
    gd = golden("ions_small.npz")
    grid = pg.Grid(tuple(int(x) for x in gd["n"]), tuple(float(x) for x in gd["L"]))
    v = grid.potential(pg.WaterTables(gd["waters"]))
    grid.add_ions(v, gd["ion_sites"], gd["ion_charges"])
    for corr in (1, 3):
        ev, _, _ = grid.solve(v, nroots=2, maxsub=20, maxiter=200, ptol=8, corrflag=corr)
        assert np.max(np.abs(np.asarray(ev) - gd["evals"][:2])) <= 1e-8, (corr, ev, gd["evals"])


def check_full_grid_against_oracle(pg, orc, grid, tables, waters, v, ions_bohr=None, ion_q=None):
    """V(r) on the whole grid against the oracle on the same site tables
    (<= 1e-13 of max|V|), and the oracle's own site producer against the
    library's (<= 1e-12); returns the oracle grid and V."""
    og = orc.Grid(grid.n, grid.L)
    vo = og.potential_dpp(tables.sites, tables.charges, tables.charge_site, tables.dipoles, tables.dipole_site)
    if ions_bohr is not None:
        og.add_ions(vo, ions_bohr.reshape(-1), ion_q)
    assert rel(host(v), vo) < 1e-13
    s = orc.dpp_sites(waters)
    assert rel(tables.sites, s[0]) < 1e-12 and rel(tables.dipoles, s[3]) < 1e-12
    return og, vo


def check_pairs_against_oracle(og, vo, evals, vecs, de_tol, res_tol):
    """Each returned pair (lambda, v) against the oracle's H (a restatement of
    src/mtx.cpp:22-109): |v.Hv / v.v - lambda| <= de_tol and
    |H v - lambda v| / |v| <= res_tol."""
    V = host(vecs)
    for r, lam in enumerate(evals):
        x = V[r]
        hx = og.matvec(vo, x)
        nrm2 = float(x @ x)
        assert abs(float(x @ hx) / nrm2 - lam) <= de_tol, (r, float(x @ hx) / nrm2, lam)
        res = float(np.linalg.norm(hx - lam * x)) / np.sqrt(nrm2)
        assert res <= res_tol, (r, res)


@pytest.mark.gpu
def test_solve_c3_against_oracle_and_fp64(pg, orc, torch, clusters):
    """c3: (H2O)32 + Na+ + Cl-, 96^3 over 48 bohr, 8 states, block 8.  V(r)
    on the full grid against the oracle (DPP + Bloomfield ions); every
    eigenpair of the FP64 form (ptol 8) and of the mixed form (ptol 6, FP64
    refinement) against the oracle's H: Rayleigh quotient within 1e-8 /
    1e-6 Eh of the eigenvalue, residual <= 10^-(ptol-1).  Mixed against FP64:
    |dE| <= 1e-6 Eh per eigenvalue, eigenvector overlap >= 1 - 1e-8."""
    import os
    orc.set_threads(os.cpu_count() or 4)
    w = clusters.water_cluster(32, 10.0, 3)
    ions = clusters.place_ions(w, 10.0, 33)
    grid = pg.Grid((96, 96, 96), (48.0, 48.0, 48.0))
    tables = pg.WaterTables(w)
    v = grid.potential(tables)
    ions_bohr = ions[:, :3] / 0.52917720859
    grid.add_ions(v, ions_bohr, ions[:, 3])
    og, vo = check_full_grid_against_oracle(pg, orc, grid, tables, w, v, ions_bohr, ions[:, 3])
    e64, x64, _ = grid.solve(v, nroots=8, maxsub=64, maxiter=400, ptol=8, corrflag=3)
    emx, xmx, _ = grid.solve(v, nroots=8, maxsub=64, maxiter=400, ptol=6, corrflag=3, precision=pg.PG_MIXED,
                             refine=1)
    check_pairs_against_oracle(og, vo, e64, x64, 1e-8, 1e-7)
    check_pairs_against_oracle(og, vo, emx, xmx, 1e-6, 1e-5)
    assert np.max(np.abs(np.asarray(emx) - np.asarray(e64))) <= 1e-6
    ov = torch.abs(torch.sum(x64 * xmx, dim=1)) / (x64.norm(dim=1) * xmx.norm(dim=1))
    assert float(ov.min()) >= 1 - 1e-8, ov
    orc.set_threads(4)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [(160, 24, 20), (24, 136, 20), (20, 24, 200), (136, 136, 8)])
def test_hx_mixed_k_chunked_axes(pg, torch, n):
    """Axes longer than 112 points run the tensor-core contraction in K
    chunks (the kinetic matrix restaged per chunk): mixed H*X against FP64
    within the mixed form's bound (2e-5 of max |Y|), on each axis."""
    rng = np.random.Generator(np.random.PCG64(6))
    grid = pg.Grid(n, tuple(0.6 * (k + 1) for k in n))
    N = grid.N
    x = dev(torch, rng.standard_normal(3 * N))
    v = dev(torch, rng.standard_normal(N))
    y64 = host(grid.hx(v, x, nvec=3, precision=0))
    ymx = host(grid.hx(v, x, nvec=3, precision=1))
    assert np.max(np.abs(ymx - y64)) / np.max(np.abs(y64)) <= 2e-5


@pytest.mark.gpu
def test_solve_c5_against_oracle_and_fp64(pg, orc, torch, clusters):
    """c5: (H2O)128 in a 14 A sphere, 160^3 over 64 bohr (4.1M points), 16
    states, block 16, maxsub 96 -- the K-chunked tensor-core path at full
    size.  V(r) on the full grid against the oracle; every eigenpair of the
    FP64 form (ptol 8) and of the mixed form (ptol 6, refine 2) against the
    oracle's H: Rayleigh quotient within 1e-8 / 1e-6 Eh, residual <=
    10^-(ptol-1).  Mixed form against the FP64 form: |dE| <= 1e-6 Eh per
    eigenvalue, eigenvector overlap >= 1 - 1e-8."""
    import os
    orc.set_threads(os.cpu_count() or 4)
    w = clusters.water_cluster(128, 14.0, 5)
    grid = pg.Grid((160, 160, 160), (64.0, 64.0, 64.0))
    tables = pg.WaterTables(w)
    v = grid.potential(tables)
    og, vo = check_full_grid_against_oracle(pg, orc, grid, tables, w, v)
    e64, x64, _ = grid.solve(v, nroots=16, maxsub=96, maxiter=400, ptol=8, corrflag=3)
    check_pairs_against_oracle(og, vo, e64, x64, 1e-8, 1e-7)
    # the FP64 Rayleigh-Ritz step fixes the eigenvalues; with states 2e-4 Eh
    # apart the vectors need the FP64 polish (refine 2) for overlap 1 - 1e-8
    emx, xmx, _ = grid.solve(v, nroots=16, maxsub=96, maxiter=400, ptol=6, corrflag=3, precision=pg.PG_MIXED,
                             refine=1)
    assert np.max(np.abs(np.asarray(emx) - np.asarray(e64))) <= 1e-6
    emx, xmx, st = grid.solve(v, nroots=16, maxsub=96, maxiter=400, ptol=6, corrflag=3, precision=pg.PG_MIXED,
                              refine=2)
    assert np.max(np.abs(np.asarray(emx) - np.asarray(e64))) <= 1e-6
    ov = torch.abs(torch.sum(x64 * xmx, dim=1)) / (x64.norm(dim=1) * xmx.norm(dim=1))
    assert float(ov.min()) >= 1 - 1e-8, ov
    check_pairs_against_oracle(og, vo, emx, xmx, 1e-6, 1e-5)
    orc.set_threads(4)


@pytest.mark.gpu
@pytest.mark.parametrize("n,nvec", [((64, 64, 64), 12), ((96, 80, 48), 6), ((112, 40, 72), 5)])
def test_hx_mixed_pipelined_many_tiles(pg, torch, n, nvec):
    """More tiles than SMs: the pipelined tensor-core form (producer warps
    fill the next tile while consumer warps drain the last accumulator)
    against FP64 within the mixed form's bound (2e-5 of max |Y|), twice in a
    row (the second launch reuses nothing of the first)."""
    rng = np.random.Generator(np.random.PCG64(8))
    grid = pg.Grid(n, tuple(0.6 * (k + 1) for k in n))
    N = grid.N
    x = dev(torch, rng.standard_normal(nvec * N))
    v = dev(torch, rng.standard_normal(N))
    y64 = host(grid.hx(v, x, nvec=nvec, precision=0))
    for _ in range(2):
        ymx = host(grid.hx(v, x, nvec=nvec, precision=1))
        assert np.max(np.abs(ymx - y64)) / np.max(np.abs(y64)) <= 2e-5
