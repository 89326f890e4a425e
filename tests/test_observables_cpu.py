"""Observables and cube files on the CPU: the oracle's restatements of the
reference's expectation values, energy partition and Small2Large against the
reference run (observables.npz), and the library's host-side cube writer and
reader against the files the reference wrote, byte for byte.

Tolerances: the printed tables match string for string (the reference
prints %10.5f); Small2Large 1e-14 relative; cube files byte-identical."""
import os
import re

import numpy as np
import pytest

from conftest import golden, rel

BOHR2ANGS = 0.52917720859          # src/constants.h:18
AU2MEV = 1000 * 27.21138386        # src/constants.h:7-8


def printed_moments(sums):
    """The reference's expectation-value table rows (src/DVR.cpp:2419-2446)
    from the per-state sums [norm, <x>, <y>, <z>, <r^2>, <n|x|0>, ...]."""
    rows, dips = [], []
    for i, s in enumerate(sums):
        rexp = np.sqrt(s[1] * s[1] + s[2] * s[2] + s[3] * s[3])
        rows.append(" %3i   %10.5f  %10.5f  %10.5f" % (i, BOHR2ANGS * rexp, BOHR2ANGS * np.sqrt(s[4]),
                                                     BOHR2ANGS * np.sqrt(s[4] - rexp * rexp)))
        if i > 0:
            d = s[5:8]
            dips.append(" %3i      %10.5f     (%10.5f,  %10.5f,  %10.5f)" % (i, d @ d, d[0], d[1], d[2]))
    return rows, dips


def printed_energies(parts):
    return [" %3i   %10.5f  %10.5f  %10.5f  %10.5f" % (i, *(AU2MEV * p)) for i, p in enumerate(parts)]


def test_oracle_expectation_values_match_reference_print(orc):
    g = golden("observables.npz")
    og = orc.Grid(g["n"], g["L"])
    ns = int(g["nconv"][0])
    sums = og.expectation_values(g["wavefn"], ns)
    text = str(g["expect_text"])
    rows, dips = printed_moments(sums)
    for line in rows + dips:
        assert line in text, (line, text)
    for i in range(ns):
        assert abs(sums[i, 0] - 1.0) < 1e-8


def test_oracle_energy_partition_matches_reference_print(orc):
    g = golden("observables.npz")
    og = orc.Grid(g["n"], g["L"])
    ns = int(g["nconv"][0])
    parts = np.concatenate([g["v_pc"], g["v_ind"], g["v_rep"], g["v_pol"]])
    e = og.energy_partition(g["wavefn"], ns, parts)
    text = str(g["energy_text"])
    for line in printed_energies(e):
        assert line in text, (line, text)


def test_oracle_small_to_large_matches_reference(orc):
    g = golden("observables.npz")
    out = orc.small_to_large(g["read_npts"], g["read_x0"], g["read_dx"], g["read_cube"], g["s2l_N"],
                             g["s2l_xmin"], g["s2l_dx"])
    assert rel(out, g["s2l"]) < 1e-14
    assert abs(float(out @ out) - 1.0) < 1e-13


def test_write_cube_is_the_reference_file(pg, tmp_path):
    g = golden("observables.npz")
    w = g["waters"].reshape(-1, 3)
    Z = np.tile([8, 1, 1], len(w) // 3)
    path = str(tmp_path / "free.cub")
    pg.write_cube(path, g["n"], g["cube_x0"], g["cube_dx"], g["state_cube"], Z=Z, pos_angstrom=w)
    assert open(path).read() == str(g["cube_free"])


def test_read_cube_reads_what_the_reference_reads(pg, tmp_path):
    g = golden("observables.npz")
    path = str(tmp_path / "StartVector.cub")
    with open(path, "w") as f:
        f.write(str(g["cube_free"]))
    npts, x0, dx, natoms, cube = pg.read_cube(path)
    assert list(npts) == list(g["read_npts"]) and natoms == 18
    assert np.array_equal(x0, g["read_x0"]) and np.array_equal(dx, g["read_dx"])
    assert np.array_equal(cube, g["read_cube"])


def test_read_cube_rejects_bad_files(pg, tmp_path):
    g = golden("observables.npz")
    text = str(g["cube_free"]).splitlines()
    bad = list(text)
    bad[3] = re.sub(r"0\.000000", "0.100000", bad[3], count=1)  # a skewed axis
    path = str(tmp_path / "skew.cub")
    open(path, "w").write("\n".join(bad) + "\n")
    with pytest.raises(pg.PiscesError) as e:
        pg.read_cube(path)
    assert e.value.status == pg.PG_BAD_ARG and "cartesian" in str(e.value)
    short = str(tmp_path / "short.cub")
    open(short, "w").write("\n".join(text[:40]) + "\n")
    with pytest.raises(pg.PiscesError):
        pg.read_cube(short)
    with pytest.raises(pg.PiscesError):
        pg.read_cube(str(tmp_path / "missing.cub"))
