"""The dual-grid single point (PolType 6) on the CPU: the oracle's
restatement of the coarse-to-fine interpolation of V and of the start
vector against the reference run (dual.npz: (H2O)6 over a 20 bohr box on
16^3, 18^3 and 20^3 points, triple spacing with 0, 1 and 2 zeroed layers,
and 17^3, double spacing; generated by tests/golden/make_golden.py from the
reference built here), and the library's coarse-grid geometry.  No GPU.

Tolerances: interpolated points and the start vector bit for bit (same
products, same order of addition); exactly evaluated points and the coarse
V relative 1e-12 of the largest |V| (the self-consistent term sums a dipole
product whose order differs)."""
import numpy as np
import pytest

from conftest import dual_exact_mask, golden, rel

GRIDS = (16, 17, 18, 20)


@pytest.fixture(scope="module")
def ref():
    return golden("dual.npz")


def pol_pos(ref):
    return ref["sites"].reshape(-1, 3)[ref["pol_site_list"]]


def poltype3_v(orc, ref, n, L):
    """V of the self-consistent model on an oracle grid: charges and Slater
    cores (no dipoles, no one-site term), then the dipole term."""
    g = orc.Grid(n, L)
    nq = len(ref["charges"])
    _, pc, ind, rep, _ = g.potential_dpp(ref["sites"], ref["charges"], ref["charge_site"], np.zeros(3 * nq),
                                         np.arange(nq, dtype=np.int32), parts=True)
    v = pc + ind + rep
    g.potential_scpol_add(v, pol_pos(ref), ref["inva"], ref["epc"], 2, 2.536, float(ref["vpol_ww"][0]))
    return g, v


@pytest.mark.parametrize("n", GRIDS)
def test_library_coarse_grid_matches_reference(pg, ref, n):
    nc, Lc, spacing = pg.dual_grid_coarse(n, 20.0)
    assert nc == tuple(int(v) for v in ref[f"coarse_n_{n}"])
    assert np.array_equal(np.array(Lc), ref[f"coarse_L_{n}"])
    assert spacing == (2 if int(ref[f"idual_{n}"][0]) == 1 else 3)


@pytest.mark.parametrize("n", GRIDS)
def test_oracle_coarse_potential_against_reference(orc, ref, n):
    nc = tuple(int(v) for v in ref[f"coarse_n_{n}"])
    _, v = poltype3_v(orc, ref, nc, tuple(float(x) for x in ref[f"coarse_L_{n}"]))
    assert rel(v, ref[f"coarse_v_{n}"]) <= 1e-12


@pytest.mark.parametrize("n", GRIDS)
def test_oracle_dual_potential_against_reference(orc, ref, n):
    g, v_exact = poltype3_v(orc, ref, (n,) * 3, (20.0,) * 3)
    nc = int(ref[f"coarse_n_{n}"][0])
    rtol = float(ref["rtol"])
    v = g.dual_potential(nc, ref["sites"], rtol, ref[f"coarse_v_{n}"], v_exact)
    vr = ref[f"v_{n}"]
    # which points were interpolated: every site farther than rtol, or on
    # the coarse lattice; the reference's value there is the interpolation
    # of its own coarse V, reproduced bit for bit
    exact = dual_exact_mask(n, nc, [g.x[a] for a in range(3)], ref["sites"], rtol)
    interp = ~exact
    assert 0 < np.count_nonzero(interp) < g.N
    assert np.array_equal(v[exact], v_exact[exact])
    assert np.array_equal(v[interp], vr[interp])
    assert rel(v, vr) <= 1e-12


@pytest.mark.parametrize("n", GRIDS)
def test_oracle_start_vector_against_reference(orc, ref, n):
    nc = int(ref[f"coarse_n_{n}"][0])
    w = orc.dual_extend(n, nc, ref[f"coarse_wavefn_{n}"])
    assert np.array_equal(w, ref[f"extended_wf_{n}"])


def test_reference_runs_converged(ref):
    for n in GRIDS:
        assert int(ref[f"coarse_nconv_{n}"][0]) == 1 and int(ref[f"nconv_{n}"][0]) == 1


def test_library_rejects_bad_dual_grids(pg):
    with pytest.raises(pg.PiscesError) as e:
        pg.dual_grid_coarse((16, 16, 18), 20.0)
    assert e.value.status == pg.PG_BAD_ARG
    with pytest.raises(pg.PiscesError) as e:
        pg.dual_grid_coarse(16, (20.0, 20.0, 22.0))
    assert e.value.status == pg.PG_BAD_ARG
