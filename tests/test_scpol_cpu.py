"""Self-consistent polarisation (PolType 3) and the Hellmann-Feynman gradient
on the CPU: the oracle's restatements against the reference run
(scpol.npz: (H2O)6 on a 14 x 16 x 18 grid, generated by
tests/golden/make_golden.py from the reference built here), and the
library's host-side pieces (the polarisable atoms, Epc and water-water
offset of a cluster; A = (alpha^-1 - T)^-1; FinalGradient) against the same
run.  No GPU.

Tolerances (relative to the largest entry): A 1e-13; V_pol, Epc and the
offset 1e-12; the grid sums of the gradient 1e-12 (the reference sums them
over OpenMP threads in a thread-count dependent order)."""
import numpy as np
import pytest

from conftest import golden, rel


@pytest.fixture(scope="module")
def ref():
    return golden("scpol.npz")


def pol_pos(ref):
    return ref["sites"].reshape(-1, 3)[ref["pol_site_list"]]


def sto_lists(pg, ref):
    t = pg.WaterTables.from_lists(ref["sites"], ref["charges"], ref["charge_site"], np.zeros(3 * len(ref["charges"])),
                                  np.arange(len(ref["charges"]), dtype=np.int32))
    sto = np.ctypeslib.as_array(t.table.sto, shape=(2 * t.table.nsto,)).copy()
    sto_site = np.ctypeslib.as_array(t.table.sto_site, shape=(t.table.nsto,)).copy()
    return sto, sto_site


def test_reference_model_layout(ref):
    # PolType 3: O, H1, H2 of every water are the polarisable atoms; no
    # induced-dipole part in V
    nw = len(ref["waters"]) // 9 if ref["waters"].ndim == 1 else len(ref["waters"])
    assert list(ref["pol_site_list"]) == [4 * j + k for j in range(nw) for k in range(3)]
    assert np.all(ref["v_ind"] == 0)
    assert int(ref["nconv"][0]) == 1


def test_oracle_inva_against_reference(orc, ref):
    A = orc.scpol_inva(pol_pos(ref), ref["alphas"])
    assert rel(A, ref["inva"].reshape(A.shape)) <= 1e-13


def test_library_inva_against_reference(pg, ref):
    A = pg.scpol_inva(pol_pos(ref), ref["alphas"])
    assert rel(A, ref["inva"].reshape(A.shape)) <= 1e-13
    assert np.array_equal(A, A.T)


def test_library_cluster_model_against_reference(pg, ref):
    # pg_water_scpol: the polarisable atoms, their polarisabilities, Epc and
    # the water-water polarisation energy of the same cluster
    m = pg.ScPol(ref["waters"])
    assert np.array_equal(m.pol_site, ref["pol_site_list"])
    assert rel(m.alpha, ref["alphas"]) <= 1e-15
    assert rel(m.epc, ref["epc"]) <= 1e-12
    assert abs(m.vpol_ww - float(ref["vpol_ww"][0])) <= 1e-12 * abs(float(ref["vpol_ww"][0]))
    assert rel(m.inva, ref["inva"].reshape(m.inva.shape)) <= 1e-12


def test_oracle_potential_against_reference(orc, ref):
    n = tuple(int(v) for v in ref["n"])
    g = orc.Grid(n, tuple(float(v) for v in ref["L"]))
    v = np.zeros(g.N)
    g.potential_scpol_add(v, pol_pos(ref), ref["inva"], ref["epc"], 2, 2.536, float(ref["vpol_ww"][0]))
    assert rel(v, ref["v_pol"]) <= 1e-12


def test_oracle_gradient_against_reference(orc, pg, ref):
    n = tuple(int(v) for v in ref["n"])
    g = orc.Grid(n, tuple(float(v) for v in ref["L"]))
    sto, sto_site = sto_lists(pg, ref)
    grad, tmu, mcm = g.hf_gradient_grid(ref["sites"], ref["charges"], ref["charge_site"], sto, sto_site,
                                        ref["pol_site_list"], ref["inva"], ref["epc"], ref["wavefn"][:g.N])
    assert rel(grad, ref["grad_grid"]) <= 1e-12
    assert np.allclose(mcm, mcm.T, rtol=0, atol=1e-15 * np.abs(mcm).max())
    total = ref["grad_ww"] + grad
    orc.hf_gradient_final(len(ref["sites"]) // 3, tmu, mcm, ref["dT_x"], ref["dT_y"], ref["dT_z"], ref["dEfield"],
                          ref["pol_grad"], total)
    assert rel(total, ref["grad_total"]) <= 1e-12


def test_library_final_gradient_matches_oracle(orc, pg, ref):
    # pg_hf_gradient_final against the oracle's FinalGradient on the same
    # (oracle) grid sums
    n = tuple(int(v) for v in ref["n"])
    g = orc.Grid(n, tuple(float(v) for v in ref["L"]))
    sto, sto_site = sto_lists(pg, ref)
    grad, tmu, mcm = g.hf_gradient_grid(ref["sites"], ref["charges"], ref["charge_site"], sto, sto_site,
                                        ref["pol_site_list"], ref["inva"], ref["epc"], ref["wavefn"][:g.N])
    ns = len(ref["sites"]) // 3
    a = ref["grad_ww"] + grad
    b = a.copy()
    orc.hf_gradient_final(ns, tmu, mcm, ref["dT_x"], ref["dT_y"], ref["dT_z"], ref["dEfield"], ref["pol_grad"], a)
    pg.hf_gradient_final(ns, tmu, mcm, ref["dT_x"], ref["dT_y"], ref["dT_z"], ref["dEfield"], ref["pol_grad"], b)
    assert rel(b, a) <= 1e-14
    assert rel(b, ref["grad_total"]) <= 1e-12


def test_library_rejects_bad_models(pg, ref):
    # not the rigid-water layout; a singular polarisation matrix
    with pytest.raises(pg.PiscesError) as e:
        pg.hf_gradient_final(10, np.zeros(9), np.zeros((9, 9)), np.zeros(81), np.zeros(81), np.zeros(81),
                             np.zeros(270), None, np.zeros(30))
    assert e.value.status == pg.PG_BAD_ARG
    with pytest.raises(pg.PiscesError) as e:
        pg.scpol_inva(np.zeros(3), [-1.0])
    assert e.value.status == pg.PG_BAD_ARG
