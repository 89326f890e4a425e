"""The reference-class shims (pisces-1_gb300/refshim): DVR::davdriver,
DVR::ComputePotential, DVR::ComputeGradient and VectorFFT compiled against
the reference's own headers and linked into the reference program in place
of its src/davdriver.cpp, its ComputePotential and ComputeGradient and its
src/VectorFFTW.cpp (oracle/ref/Makefile, target shims).  Runs where the reference tree and its
CPU build are present (the fixture-generation container); elsewhere skipped.
Checks that the link succeeds, that each of the four reference symbols is
defined once and strongly (by the shim, not the reference), and that the
calls they make resolve to libpisces_gb300.so."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(ROOT, "oracle", "_ref")
EXE = os.path.join(OUT, "pisces_ref_gb300")


def _have_reference():
    import __graft_entry__ as entry
    return os.path.isdir(os.path.join(entry.REFERENCE_TREE, "src")) and os.path.exists(
        os.path.join(OUT, "pisces_ref"))


@pytest.mark.skipif(not _have_reference(), reason="needs the reference tree and its CPU build (oracle/_ref)")
def test_shims_link_into_the_reference(pg):
    import __graft_entry__ as entry
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={entry.REFERENCE_TREE}",
                        "shims"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    syms = subprocess.run(["nm", "-C", EXE], capture_output=True, text=True, check=True).stdout.splitlines()
    for name in ("DVR::davdriver(int, int, int, int, int, int, double*)", "DVR::ComputePotential(Potential&)",
                 "DVR::ComputeGradient(Potential&, int, double*, double*, double*, double*, double*, WaterCluster&, "
                 "double*)",
                 "VectorFFT::apply(double const*, double*, double const*, double const*)"):
        defs = [s for s in syms if s.endswith(" " + name)]
        assert len(defs) == 1 and " T " in defs[0], (name, defs)
    shim_objs = os.path.join(OUT, "shim_obj")
    for obj, name in (("davdriver_gb300.o", "DVR::davdriver"), ("computepotential_gb300.o", "DVR::ComputePotential"),
                      ("computegradient_gb300.o", "DVR::ComputeGradient"), ("vectorfft_gb300.o", "VectorFFT::apply")):
        own = subprocess.run(["nm", "-C", os.path.join(shim_objs, obj)], capture_output=True, text=True,
                             check=True).stdout
        assert any(" T " + name in line for line in own.splitlines()), (obj, name)
    undef = subprocess.run(["nm", "-D", "--undefined-only", EXE], capture_output=True, text=True,
                           check=True).stdout
    calls = ("pg_solve", "pg_grid_create_dvr", "pg_potential_eval", "pg_hx", "pg_potential_scpol_add",
             "pg_hf_gradient_grid", "pg_hf_gradient_final", "pg_dual_grid_potential")
    for call in calls:
        assert f" {call}" in undef, call
    needed = subprocess.run(["readelf", "-d", EXE], capture_output=True, text=True, check=True).stdout
    assert "libpisces_gb300.so" in needed
    exported = subprocess.run(["nm", "-D", "--defined-only", pg.LIB_PATH], capture_output=True, text=True,
                              check=True).stdout
    for call in calls:
        assert f" T {call}" in exported, call
