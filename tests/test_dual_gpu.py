"""The dual-grid single point (PolType 6) on the GPU against the reference
run (dual.npz: (H2O)6 over a 20 bohr box on 16^3, 18^3 and 20^3 points,
triple spacing with 0, 1 and 2 zeroed layers, and 17^3, double spacing;
Rtol 6 bohr) and the oracle.

- pg_dual_grid_potential from the reference's coarse V: the interpolated
  points bit for bit (same products, same order of addition; the file is
  built without contraction), every point within 1e-12 of the largest |V|
  (the exact points carry the self-consistent dipole term, summed in
  another order), the exact-point count equal to the oracle's.
- pg_dual_grid_extend from the reference's coarse ground state: bit for bit.
- The whole single point through the library (coarse V and solve, fine V,
  interpolated start, fine solve): coarse and fine ground-state energies
  within 1e-9 Eh of the reference's.
- A 64^3 grid of (H2O)24 (triple spacing: n = 64 gives 22 coarse points)
  against the oracle, with several thousand exact points.
- Bit for bit run to run; bad coarse sizes are PG_BAD_ARG."""
import numpy as np
import pytest

from conftest import dual_exact_mask, golden, rel

pytestmark = pytest.mark.gpu

GRIDS = (16, 17, 18, 20)


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


@pytest.fixture(scope="module")
def ref():
    return golden("dual.npz")


def ref_model(pg, ref):
    nq = len(ref["charges"])
    t = pg.WaterTables.from_lists(ref["sites"], ref["charges"], ref["charge_site"], np.zeros(3 * nq),
                                  np.arange(nq, dtype=np.int32))
    return pg.ScPol(tables=t, pol_site=ref["pol_site_list"], inva=ref["inva"], epc=ref["epc"],
                    vpol_ww=float(ref["vpol_ww"][0]))


def oracle_dual(orc, ref, n, nc, v_coarse, rtol):
    g = orc.Grid((n,) * 3, (20.0,) * 3)
    nq = len(ref["charges"])
    _, pc, ind, rep, _ = g.potential_dpp(ref["sites"], ref["charges"], ref["charge_site"], np.zeros(3 * nq),
                                         np.arange(nq, dtype=np.int32), parts=True)
    v_exact = pc + ind + rep
    pos = ref["sites"].reshape(-1, 3)[ref["pol_site_list"]]
    g.potential_scpol_add(v_exact, pos, ref["inva"], ref["epc"], 2, 2.536, float(ref["vpol_ww"][0]))
    v = g.dual_potential(nc, ref["sites"], rtol, v_coarse, v_exact)
    return v, v_exact


@pytest.mark.parametrize("n", GRIDS)
def test_dual_potential_matches_reference(pg, orc, torch, ref, n):
    nc = int(ref[f"coarse_n_{n}"][0])
    grid = pg.Grid(n, 20.0)
    vc = torch.from_numpy(ref[f"coarse_v_{n}"].copy()).cuda()
    v, n_exact = grid.dual_potential(nc, vc, ref_model(pg, ref), float(ref["rtol"]))
    vh = v.cpu().numpy()
    vr = ref[f"v_{n}"]
    vo, _ = oracle_dual(orc, ref, n, nc, ref[f"coarse_v_{n}"], float(ref["rtol"]))
    interp = ~dual_exact_mask(n, nc, grid.points(), ref["sites"], float(ref["rtol"]))
    assert n_exact == grid.N - np.count_nonzero(interp)
    assert 0 < n_exact < grid.N
    assert np.array_equal(vh[interp], vr[interp])
    assert rel(vh, vr) <= 1e-12
    assert rel(vh, vo) <= 1e-12
    v2, _ = grid.dual_potential(nc, vc, ref_model(pg, ref), float(ref["rtol"]))
    assert torch.equal(v, v2)


@pytest.mark.parametrize("n", GRIDS)
def test_dual_start_vector_matches_reference(pg, torch, ref, n):
    nc = int(ref[f"coarse_n_{n}"][0])
    grid = pg.Grid(n, 20.0)
    wc = torch.from_numpy(ref[f"coarse_wavefn_{n}"].copy()).cuda()
    w = grid.dual_extend(nc, wc).cpu().numpy()
    assert np.array_equal(w, ref[f"extended_wf_{n}"])


@pytest.mark.parametrize("n", GRIDS)
def test_dual_single_point_matches_reference(pg, torch, ref, n):
    r = pg.dual_single_point(n, 20.0, ref_model(pg, ref), rtol=float(ref["rtol"]), nroots=1, maxsub=20, maxiter=300,
                             ptol=8)
    assert r["coarse_n"] == tuple(int(v) for v in ref[f"coarse_n_{n}"])
    assert abs(r["coarse_evals"][0] - float(ref[f"coarse_evals_{n}"][0])) <= 1e-9
    assert abs(r["evals"][0] - float(ref[f"evals_{n}"][0])) <= 1e-9, (r["evals"], ref[f"evals_{n}"])
    assert rel(r["v"].cpu().numpy(), ref[f"v_{n}"]) <= 1e-12


def test_dual_potential_64_against_oracle(pg, orc, torch, clusters):
    # (H2O)24 over 40 bohr; n = 64 -> 22 coarse points, triple spacing;
    # Rtol 4 bohr
    w = clusters.water_cluster(24, 9.0, 2)
    model = pg.ScPol(w)
    n, L, rtol = 64, 40.0, 4.0
    nc, Lc, spacing = pg.dual_grid_coarse(n, L)
    assert nc == (22, 22, 22) and spacing == 3
    coarse = pg.Grid(nc, Lc)
    vc = coarse.potential_scpol(model)
    grid = pg.Grid(n, L)
    v, n_exact = grid.dual_potential(nc, vc, model, rtol)
    t = model.table
    sites = np.ctypeslib.as_array(t.sites, shape=(3 * t.nsites,)).copy()
    q = np.ctypeslib.as_array(t.charges, shape=(t.ncharges,)).copy()
    qs = np.ctypeslib.as_array(t.charge_site, shape=(t.ncharges,)).copy()
    g = orc.Grid((n,) * 3, (L,) * 3)
    _, pc, ind, rep, _ = g.potential_dpp(sites, q, qs, np.zeros(3 * len(q)), np.arange(len(q), dtype=np.int32),
                                         parts=True)
    v_exact = pc + ind + rep
    g.potential_scpol_add(v_exact, sites.reshape(-1, 3)[model.pol_site], model.inva, model.epc, 2, 2.536,
                          model.vpol_ww)
    vo = g.dual_potential(nc[0], sites, rtol, vc.cpu().numpy(), v_exact)
    interp = ~dual_exact_mask(n, nc[0], grid.points(), sites, rtol)
    assert n_exact == grid.N - np.count_nonzero(interp) and n_exact > 1000
    vh = v.cpu().numpy()
    assert np.array_equal(vh[interp], vo[interp])
    assert rel(vh, vo) <= 1e-12
    wc = torch.randn(coarse.N, dtype=torch.float64, device="cuda")
    assert np.array_equal(grid.dual_extend(nc, wc).cpu().numpy(), orc.dual_extend(n, nc[0], wc.cpu().numpy()))


def test_dual_rejects_bad_sizes(pg, torch):
    grid = pg.Grid(16, 20.0)
    vc = torch.zeros(7 ** 3, dtype=torch.float64, device="cuda")
    with pytest.raises(pg.PiscesError) as e:
        grid.dual_extend(7, vc)
    assert e.value.status == pg.PG_BAD_ARG
    g2 = pg.Grid((16, 16, 18), 20.0)
    with pytest.raises(pg.PiscesError) as e:
        g2.dual_extend(6, vc)
    assert e.value.status == pg.PG_BAD_ARG
