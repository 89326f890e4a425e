"""Self-consistent polarisation (PolType 3) and the Hellmann-Feynman gradient
on the GPU.

- Against the reference run (scpol.npz, (H2O)6 on 16^3 points over a
  20 x 22 x 24 bohr box): V and its four parts from the reference's own
  model tables (relative 1e-13) and from the library's own host pipeline
  (1e-12); the ground-state energy of the FP64 solve on that V (1e-9 Eh);
  the gradient's grid sums for the reference's ground state, and the full
  gradient with the reference's water-side inputs (1e-12).
- Against the oracle at larger sizes: (H2O)24 on 40^3 points (V on the full
  grid, 1e-12) and 24^3 (gradient sums, 1e-12); and a 96^3 grid whose dipole
  products run in two chunks of points (V at sampled points against a numpy
  evaluation; the gradient for a sparse density against the oracle).
- Bit for bit run to run."""
import numpy as np
import pytest

from conftest import golden, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


@pytest.fixture(scope="module")
def ref():
    return golden("scpol.npz")


def ref_model(pg, ref):
    t = pg.WaterTables.from_lists(ref["sites"], ref["charges"], ref["charge_site"], np.zeros(3 * len(ref["charges"])),
                                  np.arange(len(ref["charges"]), dtype=np.int32))
    return pg.ScPol(tables=t, pol_site=ref["pol_site_list"], inva=ref["inva"], epc=ref["epc"],
                    vpol_ww=float(ref["vpol_ww"][0]))


def grid_of(pg, ref):
    return pg.Grid(tuple(int(v) for v in ref["n"]), tuple(float(v) for v in ref["L"]))


def test_potential_matches_reference(pg, torch, ref):
    grid = grid_of(pg, ref)
    v, parts = grid.potential_scpol(ref_model(pg, ref), parts=True)
    torch.cuda.synchronize()
    assert rel(v.cpu().numpy(), ref["v"]) <= 1e-13
    p = parts.cpu().numpy()
    for k, name in enumerate(("v_pc", "v_ind", "v_rep", "v_pol")):
        assert rel(p[k], ref[name]) <= 1e-13 if name != "v_ind" else np.all(p[k] == 0), name
    # the library's own model of the same waters
    v2 = grid.potential_scpol(pg.ScPol(ref["waters"]))
    assert rel(v2.cpu().numpy(), ref["v"]) <= 1e-12
    # bit for bit run to run
    assert torch.equal(grid.potential_scpol(ref_model(pg, ref)), v)


def test_solve_on_scpol_potential_matches_reference(pg, torch, ref):
    grid = grid_of(pg, ref)
    v = grid.potential_scpol(ref_model(pg, ref))
    ev, vec, st = grid.solve(v, nroots=1, ptol=8, maxsub=20, maxiter=300)
    assert abs(ev[0] - float(ref["evals"][0])) <= 1e-9, (ev, ref["evals"])


def test_gradient_matches_reference(pg, torch, ref):
    grid = grid_of(pg, ref)
    m = ref_model(pg, ref)
    psi = torch.from_numpy(ref["wavefn"][:grid.N].copy()).cuda()
    grad, tmu, mcm = grid.hf_gradient_grid(m, psi)
    assert rel(grad, ref["grad_grid"]) <= 1e-12
    assert np.array_equal(mcm, mcm.T)
    total = ref["grad_ww"] + grad
    pg.hf_gradient_final(len(ref["sites"]) // 3, tmu, mcm, ref["dT_x"], ref["dT_y"], ref["dT_z"],
                         ref["dEfield"], ref["pol_grad"], total)
    assert rel(total, ref["grad_total"]) <= 1e-12
    g2, t2, m2 = grid.hf_gradient_grid(m, psi)
    assert np.array_equal(g2, grad) and np.array_equal(t2, tmu) and np.array_equal(m2, mcm)


def lists(pg, model):
    t = model.table
    sites = np.ctypeslib.as_array(t.sites, shape=(3 * t.nsites,)).copy()
    q = np.ctypeslib.as_array(t.charges, shape=(t.ncharges,)).copy()
    qs = np.ctypeslib.as_array(t.charge_site, shape=(t.ncharges,)).copy()
    sto = np.ctypeslib.as_array(t.sto, shape=(2 * t.nsto,)).copy()
    ss = np.ctypeslib.as_array(t.sto_site, shape=(t.nsto,)).copy()
    return sites, q, qs, sto, ss


@pytest.fixture(scope="module")
def w24(clusters):
    return clusters.water_cluster(24, 9.0, 2)


def test_potential_c2_cluster_against_oracle(pg, orc, torch, w24):
    n, L = (40, 40, 40), (40.0, 40.0, 40.0)
    m = pg.ScPol(w24)
    grid = pg.Grid(n, L)
    v = torch.zeros(grid.N, dtype=torch.float64, device="cuda")
    grid.scpol_add(m, v)
    g = orc.Grid(n, L)
    sites = lists(pg, m)[0]
    vo = g.potential_scpol_add(np.zeros(g.N), sites.reshape(-1, 3)[m.pol_site], m.inva, m.epc, 2, 2.536, m.vpol_ww)
    assert rel(v.cpu().numpy(), vo) <= 1e-12


def test_gradient_c2_cluster_against_oracle(pg, orc, torch, w24):
    n, L = (24, 24, 24), (40.0, 40.0, 40.0)
    m = pg.ScPol(w24)
    grid = pg.Grid(n, L)
    psi = grid.piab()
    grad, tmu, mcm = grid.hf_gradient_grid(m, psi)
    sites, q, qs, sto, ss = lists(pg, m)
    g = orc.Grid(n, L)
    go, to, mo = g.hf_gradient_grid(sites, q, qs, sto, ss, m.pol_site, m.inva, m.epc, psi.cpu().numpy())
    assert rel(grad, go) <= 1e-12
    assert rel(tmu, to) <= 1e-12
    assert rel(mcm, mo) <= 1e-12


def test_two_chunks_on_96_grid(pg, orc, torch, w24):
    # 96^3 points x 216 dipole components: E does not fit one 1 GiB chunk
    n, L = (96, 96, 96), (48.0, 48.0, 48.0)
    m = pg.ScPol(w24)
    grid = pg.Grid(n, L)
    v = torch.zeros(grid.N, dtype=torch.float64, device="cuda")
    grid.scpol_add(m, v)
    vh = v.cpu().numpy()
    rng = np.random.Generator(np.random.PCG64(96))
    idx = np.sort(rng.choice(grid.N, size=600, replace=False))
    idx = np.concatenate([idx, [0, grid.N // 2, grid.N // 2 + 1, grid.N - 1]])
    xs = grid.points()
    sites = lists(pg, m)[0]
    pos = sites.reshape(-1, 3)[m.pol_site]
    ix, iy, iz = idx % n[0], (idx // n[0]) % n[1], idx // (n[0] * n[1])
    r = np.stack([xs[0][ix], xs[1][iy], xs[2][iz]], axis=1)
    d = r[:, None, :] - pos[None, :, :]
    R = np.sqrt((d * d).sum(-1))
    gfac = 1.0 / (R ** 3)
    q = R / 2.536
    reff = 2.536 * (0.5 + q ** 3 * (1.0 - 0.5 * q))
    gfac = np.where(R < 2.536, 1.0 / reff ** 3, gfac)
    E = (gfac[..., None] * d).reshape(len(idx), -1) + m.epc[None, :]
    want = -0.5 * np.einsum("pi,ij,pj->p", E, m.inva, E) - m.vpol_ww
    assert rel(vh[idx], want) <= 1e-12
    # gradient for a sparse density spread over both chunks, against the oracle
    psi = np.zeros(grid.N)
    sp = rng.choice(grid.N, size=1500, replace=False)
    psi[sp] = rng.standard_normal(len(sp))
    grad, tmu, mcm = grid.hf_gradient_grid(m, torch.from_numpy(psi).cuda())
    sites, qq, qs, sto, ss = lists(pg, m)
    go, to, mo = orc.Grid(n, L).hf_gradient_grid(sites, qq, qs, sto, ss, m.pol_site, m.inva, m.epc, psi)
    assert rel(grad, go) <= 1e-12
    assert rel(tmu, to) <= 1e-12
    assert rel(mcm, mo) <= 1e-12
