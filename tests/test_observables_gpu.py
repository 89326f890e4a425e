"""Observables and cube files of converged states on the device, against the
reference run (observables.npz: (H2O)6, 14^3 over 20 bohr, three states) and
the oracle.

Tolerances: moments and energy partition 1e-13 relative to the oracle and
the reference's printed tables string for string; the state cube bit for
bit; cube files byte for byte; Small2Large 1e-13 relative."""
import numpy as np
import pytest

from conftest import golden, rel
from test_observables_cpu import printed_energies, printed_moments

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def dev(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def test_expectation_values(pg, orc, torch):
    g = golden("observables.npz")
    ns = int(g["nconv"][0])
    grid = pg.Grid(g["n"], g["L"])
    m = grid.expectation_values(dev(torch, g["wavefn"]), ns)
    got = np.array([[d["norm"], *d["r"], d["r2"], *d["trans_dipole"]] for d in m])
    ref = orc.Grid(g["n"], g["L"]).expectation_values(g["wavefn"], ns)
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    rows, dips = printed_moments(got)
    for line in rows + dips:
        assert line in str(g["expect_text"]), line


def test_energy_partition(pg, orc, torch):
    g = golden("observables.npz")
    ns = int(g["nconv"][0])
    grid = pg.Grid(g["n"], g["L"])
    parts = np.concatenate([g["v_pc"], g["v_ind"], g["v_rep"], g["v_pol"]])
    e = grid.energy_partition(dev(torch, g["wavefn"]), dev(torch, parts), ns)
    ref = orc.Grid(g["n"], g["L"]).energy_partition(g["wavefn"], ns, parts)
    assert np.max(np.abs(e - ref)) <= 1e-13 * np.max(np.abs(ref))
    for line in printed_energies(e):
        assert line in str(g["energy_text"]), line
    # the same with V and its parts from the library's own potential
    v, p = grid.potential(pg.WaterTables(g["waters"]), parts=True)
    e2 = grid.energy_partition(dev(torch, g["wavefn"]), p.reshape(-1).contiguous(), ns)
    assert np.max(np.abs(e2 - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_state_cube_and_cube_files(pg, torch, tmp_path):
    g = golden("observables.npz")
    grid = pg.Grid(g["n"], g["L"])
    N = grid.N
    wf = g["wavefn"].reshape(-1, N)
    assert np.array_equal(grid.state_cube(wf[0]), g["state_cube"])
    w = g["waters"].reshape(-1, 3)
    Z = np.tile([8, 1, 1], len(w) // 3)
    p1 = str(tmp_path / "gauss.cub")
    integral = grid.write_state_cube(p1, wf[0], iwf=1, Z=Z, pos_angstrom=w, cubeflag=0)
    assert open(p1).read() == str(g["cube_gauss"])
    assert abs(integral - 1.0) < 1e-8
    last = int(g["cube_gomol_state"][0])
    p2 = str(tmp_path / "gomol.cub")
    grid.write_state_cube(p2, wf[last - 1], iwf=last, Z=Z, pos_angstrom=w, cubeflag=1)
    assert open(p2).read() == str(g["cube_gomol"])
    # the orbital cube reads back (negative atom count, orbital line skipped)
    npts, x0, dx, natoms, cube = pg.read_cube(p1)
    assert natoms == -len(Z) and list(npts) == list(g["n"])
    assert np.max(np.abs(cube - g["state_cube"])) <= 5e-7 * np.max(np.abs(g["state_cube"]))


def test_small_to_large(pg, orc, torch):
    g = golden("observables.npz")
    N, L = tuple(int(v) for v in g["s2l_N"]), tuple(float(v) for v in g["L"])
    big = pg.Grid(N, L)
    wf = big.small_to_large(g["read_npts"], g["read_x0"], g["read_dx"], g["read_cube"])
    assert rel(wf.cpu().numpy(), g["s2l"]) < 1e-13
    assert abs(float((wf * wf).sum()) - 1.0) < 1e-13
    # a start vector made so converges like the reference's own start vectors
    v = big.potential(pg.WaterTables(g["waters"]))
    ev, _, st = big.solve(v, nroots=1, ptol=7, maxsub=30, maxiter=300, start=wf)
    ev0, _, st0 = big.solve(v, nroots=1, ptol=7, maxsub=30, maxiter=300)
    assert abs(ev[0] - ev0[0]) < 1e-9
