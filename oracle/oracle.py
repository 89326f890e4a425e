"""ctypes front end of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE.

Only the test suite, the smoke check and the CPU-baseline leg of the bench
import this module, and only as the checker or as the timed CPU baseline.
The product library never imports, links or falls back to anything here.

Also reads the record files written by the reference driver
(oracle/ref/ref_driver.cpp) and runs that driver when it has been built
(oracle/_ref/pisces_ref, present only where the reference tree was).
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "pisces_ref")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build(quiet: bool = True) -> str:
    """Compile liboracle.so from pisces_oracle.c (gcc + OpenMP)."""
    src = os.path.join(HERE, "pisces_oracle.c")
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB_PATH, src, "-lm"]
    subprocess.run(cmd, check=True, capture_output=quiet)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(HERE, "pisces_oracle.c")
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
            build()
        L = C.CDLL(LIB_PATH)
        L.or_sine_dvr.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, _dp, _dp]
        L.or_matvec.argtypes = [_ip, C.POINTER(_dp), _dp, _dp, _dp]
        L.or_diagonal.argtypes = [_ip, C.POINTER(_dp), _dp, _dp]
        L.or_piab_start.argtypes = [_ip, C.POINTER(_dp), _dp]
        L.or_dpp_sites.argtypes = [C.c_int, _dp, _dp, _dp, _ip, _dp, _ip]
        L.or_dpp_sites.restype = C.c_int
        L.or_potential_ions_add.argtypes = [_ip, C.POINTER(_dp), C.c_int, _dp, _dp, C.c_double, C.c_double, _dp]
        L.or_potential_spherical.argtypes = [_ip, C.POINTER(_dp), C.c_double, _dp]
        L.or_solve.argtypes = [_ip, C.POINTER(_dp), C.POINTER(_dp), _dp, C.c_int, C.c_int, C.c_int, C.c_int,
                               C.c_int, C.c_int, _dp, _dp, C.POINTER(C.c_long), C.c_long]
        L.or_solve.restype = C.c_int
        L.or_syev.argtypes = [C.c_int, _dp, C.c_int, _dp, _dp, C.c_int]
        L.or_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def set_threads(n: int):
    """OpenMP thread count of the oracle's loops (the results do not depend on it)."""
    lib().or_set_threads(int(n))


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class _Tables(C.Structure):
    _fields_ = [("nsites", C.c_int), ("sites", _dp),
                ("ncharges", C.c_int), ("charges", _dp), ("charge_site", _ip),
                ("ndipoles", C.c_int), ("dipoles", _dp), ("dipole_site", _ip),
                ("nsto", C.c_int), ("sto", _dp), ("sto_site", _ip),
                ("npol", C.c_int), ("pol_alpha", _dp), ("pol_site", _ip),
                ("charge_damp", C.c_double), ("dipole_damp", C.c_double), ("pol_damp", C.c_double)]


def sine_dvr(n: int, L: float):
    x = np.empty(n)
    t = np.empty(n * (n + 1) // 2)
    lib().or_sine_dvr(n, 1.0, -0.5 * L, 0.5 * L, _d(x), _d(t))
    return x, t


def unpack(tp: np.ndarray, n: int) -> np.ndarray:
    T = np.zeros((n, n))
    a, b = np.tril_indices(n)
    T[a, b] = tp
    T[b, a] = tp
    return T


class Grid:
    """Sine-DVR grid in the reference convention (walls at -L/2, +L/2)."""

    def __init__(self, n, L):
        self.n = np.ascontiguousarray(n, dtype=np.int32)
        self.L = np.asarray(L, dtype=np.float64)
        self.x, self.tp = [], []
        for a in range(3):
            xa, ta = sine_dvr(int(self.n[a]), float(self.L[a]))
            self.x.append(xa)
            self.tp.append(ta)
        self._tp_ptrs = (_dp * 3)(*[_d(t) for t in self.tp])
        self._x_ptrs = (_dp * 3)(*[_d(t) for t in self.x])

    @property
    def N(self):
        return int(np.prod(self.n))

    def matvec(self, v, x):
        y = np.empty(self.N)
        lib().or_matvec(_i(self.n), self._tp_ptrs, _d(v), _d(np.ascontiguousarray(x)), _d(y))
        return y

    def diagonal(self, v):
        d = np.empty(self.N)
        lib().or_diagonal(_i(self.n), self._tp_ptrs, _d(v), _d(d))
        return d

    def piab(self):
        w = np.empty(self.N)
        lib().or_piab_start(_i(self.n), self._x_ptrs, _d(w))
        return w

    def potential_dpp(self, sites, charges, charge_site, dipoles, dipole_site, parts=False):
        """Default DPPGTOP model V on the grid from the water-site tables."""
        nw = len(sites) // 12
        sites = np.ascontiguousarray(sites, dtype=np.float64)
        charges = np.ascontiguousarray(charges, dtype=np.float64)
        charge_site = np.ascontiguousarray(charge_site, dtype=np.int32)
        dipoles = np.ascontiguousarray(dipoles, dtype=np.float64)
        dipole_site = np.ascontiguousarray(dipole_site, dtype=np.int32)
        sto = np.empty(8 * nw)
        sto_site = np.empty(4 * nw, dtype=np.int32)
        pa = np.empty(nw)
        ps = np.empty(nw, dtype=np.int32)
        t = _Tables()
        L = lib()
        L.or_dpp_default_tables.argtypes = [C.c_int, _dp, _dp, _ip, _dp, _ip, _dp, _ip, _dp, _ip, C.POINTER(_Tables)]
        L.or_dpp_default_tables(nw, _d(sites), _d(charges), _i(charge_site), _d(dipoles), _i(dipole_site),
                                _d(sto), _i(sto_site), _d(pa), _i(ps), C.byref(t))
        v = np.empty(self.N)
        out = [np.empty(self.N) for _ in range(4)]
        L.or_potential_dpp.argtypes = [_ip, C.POINTER(_dp), C.POINTER(_Tables), _dp, _dp, _dp, _dp, _dp]
        L.or_potential_dpp(_i(self.n), self._x_ptrs, C.byref(t), _d(v), *[_d(o) for o in out])
        return (v, *out) if parts else v

    def add_ions(self, v, pos_bohr, q, r_cation=2.9, r_anion=1.0):
        pos = np.ascontiguousarray(pos_bohr, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        lib().or_potential_ions_add(_i(self.n), self._x_ptrs, len(q), _d(pos), _d(q), r_cation, r_anion, _d(v))
        return v

    def spherical(self, k):
        v = np.empty(self.N)
        lib().or_potential_spherical(_i(self.n), self._x_ptrs, float(k), _d(v))
        return v

    def expectation_values(self, wf, nstates):
        """Sums of psi^2 (1, x, y, z, r^2) and psi_n x psi_0 per state (DVR::ExpectationValues): [nstates, 8]."""
        out = np.empty(8 * nstates)
        L = lib()
        L.or_expectation_values.argtypes = [_ip, C.POINTER(_dp), _dp, C.c_int, _dp]
        L.or_expectation_values(_i(self.n), self._x_ptrs, _d(np.ascontiguousarray(wf, dtype=np.float64)), nstates,
                                _d(out))
        return out.reshape(nstates, 8)

    def energy_partition(self, wf, nstates, parts):
        """Sums of psi^2 times the four potential parts per state (DVR::EnergyPartitioning): [nstates, 4]."""
        out = np.empty(4 * nstates)
        L = lib()
        L.or_energy_partition.argtypes = [_ip, _dp, C.c_int, _dp, _dp]
        L.or_energy_partition(_i(self.n), _d(np.ascontiguousarray(wf, dtype=np.float64)), nstates,
                              _d(np.ascontiguousarray(parts, dtype=np.float64)), _d(out))
        return out.reshape(nstates, 4)

    def potential_scpol_add(self, v, pos, inva, epc, damp_type=2, damp=2.536, vww=0.0):
        """v += -1/2 E.(A E) - vww point by point (or_potential_scpol_add)."""
        L = lib()
        L.or_potential_scpol_add.argtypes = [_ip, C.POINTER(_dp), C.c_int, _dp, _dp, _dp, C.c_int, C.c_double,
                                             C.c_double, _dp]
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        inva = np.ascontiguousarray(inva, dtype=np.float64)
        epc = np.ascontiguousarray(epc, dtype=np.float64).reshape(-1)
        L.or_potential_scpol_add(_i(self.n), self._x_ptrs, len(pos) // 3, _d(pos), _d(inva), _d(epc), int(damp_type),
                                 float(damp), float(vww), _d(v))
        return v

    def hf_gradient_grid(self, sites, charges, charge_site, sto, sto_site, pol_site, inva, epc, psi,
                         charge_damp=1.7724, pol_damp=2.536):
        """(grad, tmu, mcm): the density-weighted grid sums (or_hf_gradient_grid)."""
        L = lib()
        L.or_hf_gradient_grid.argtypes = [_ip, C.POINTER(_dp), C.c_int, _dp, C.c_int, _dp, _ip, C.c_double, C.c_int,
                                          _dp, _ip, C.c_int, _ip, _dp, _dp, C.c_double, _dp, _dp, _dp, _dp]
        a = lambda x, t=np.float64: np.ascontiguousarray(x, dtype=t).reshape(-1)
        sites, charges, sto, inva, epc, psi = a(sites), a(charges), a(sto), a(inva), a(epc), a(psi)
        charge_site, sto_site, pol_site = a(charge_site, np.int32), a(sto_site, np.int32), a(pol_site, np.int32)
        ns, npp = len(sites) // 3, len(pol_site)
        grad, tmu, mcm = np.empty(3 * ns), np.empty(3 * npp), np.empty((3 * npp, 3 * npp))
        L.or_hf_gradient_grid(_i(self.n), self._x_ptrs, ns, _d(sites), len(charges), _d(charges), _i(charge_site),
                              float(charge_damp), len(sto) // 2, _d(sto), _i(sto_site), npp, _i(pol_site), _d(inva),
                              _d(epc), float(pol_damp), _d(psi), _d(grad), _d(tmu), _d(mcm))
        return grad, tmu, mcm

    def dual_potential(self, nc, sites, rtol, v_coarse, v_exact):
        """PolType 6 V from the exact fine V and the coarse V (or_dual_potential)."""
        L = lib()
        L.or_dual_potential.argtypes = [C.c_int, C.c_int, C.POINTER(_dp), C.c_int, _dp, C.c_double, _dp, _dp, _dp]
        sites = np.ascontiguousarray(sites, dtype=np.float64).reshape(-1)
        vc = np.ascontiguousarray(v_coarse, dtype=np.float64)
        ve = np.ascontiguousarray(v_exact, dtype=np.float64)
        v = np.empty(self.N)
        L.or_dual_potential(int(self.n[0]), int(nc), self._x_ptrs, len(sites) // 3, _d(sites), float(rtol), _d(vc),
                            _d(ve), _d(v))
        return v

    def solve(self, v, nstates=1, maxsub=20, maxiter=100, ptol=5, corrflag=1, startvec=1, max_matvec=0):
        """Reference-algorithm Davidson; returns (status, evals, vectors, n_matvec)."""
        ev = np.zeros(nstates)
        B = np.zeros(self.N * maxsub)
        nmv = C.c_long(0)
        st = lib().or_solve(_i(self.n), self._tp_ptrs, self._x_ptrs, _d(np.ascontiguousarray(v)), nstates, maxsub,
                            maxiter, ptol, corrflag, startvec, _d(ev), _d(B), C.byref(nmv), int(max_matvec))
        return st, ev, B[: self.N * nstates].reshape(nstates, self.N), nmv.value


# ------------------------------------------------------------ FFT kinetic path
# numpy restatement of the reference's DVRType 3 (periodic FFT kinetic term),
# numpy's FFT standing in for FFTW (the same unnormalised forward / backward
# pair up to numpy's 1/N on the inverse).  FFTW is not part of the reference
# tree; the oracle build of the reference links a DFT computed from its
# definition in its place (oracle/ref/shim/shim.c), so the reference's own
# DVR::SetupDVR (type 3) and VectorFFT::apply run, and this restatement is
# pinned against them (tests/golden/fft.npz, test_fft_path_matches_reference_run).

REF_PI = 3.14159265358979  # src/KE_diag.cpp:28-30


def fft_tdiag(n: int, mu: float, x0: float, xNp1: float):
    """Tdiag (src/KE_diag.cpp:33-80): interior grid points and plane-wave
    energies (dK kpoint)^2 / (2 mu), dK = 2 f2 / dx, f2 = pi / n."""
    dx = (xNp1 - x0) / (n + 1)
    x = np.array([x0 + dx * (j + 1) for j in range(n)])
    f2 = REF_PI / n
    dk = 2.0 * f2 / dx
    e = np.empty(n)
    for a in range(n):
        kp = a - n if a >= n // 2 else a
        e[a] = (dk * kp) ** 2 / (2.0 * mu)
    return x, e


def fft_ke_diag(n3, L3):
    """KE_diag[xa1*n1*n2 + ya2*n2 + za3] = e0[xa1] + e1[ya2] + e2[za3]
    (src/DVR.cpp:617-630), with e_a from Tdiag on the walls -L/2, L/2."""
    e = [fft_tdiag(int(n3[a]), 1.0, -0.5 * L3[a], 0.5 * L3[a])[1] for a in range(3)]
    return (e[0][:, None, None] + e[1][None, :, None] + e[2][None, None, :]).reshape(-1)


def fft_apply(x, v_diag, n3, ke_diag):
    """VectorFFT::apply (src/VectorFFTW.cpp:56-112): y = V x + ifft(K fft(x)) / N.
    FFTW's 3-D r2c sees the array as [n0][n1][n2] (n2 fastest, dims
    n_1dbas); the half spectrum element [i][j] (i over n0*n1, j < n2/2+1) is
    multiplied by KE_diag[ng*i + j] with ng = n_1dbas[0] (cubic grids)."""
    n0, n1, n2 = (int(a) for a in n3)
    ng = n0
    ng_h = n2 // 2 + 1
    phi = np.fft.rfftn(np.asarray(x, dtype=np.float64).reshape(n0, n1, n2))
    flat = phi.reshape(n0 * n1, ng_h)
    idx = ng * np.arange(n0 * n1)[:, None] + np.arange(ng_h)[None, :]
    flat *= np.asarray(ke_diag)[idx]
    back = np.fft.irfftn(flat.reshape(n0, n1, ng_h), s=(n0, n1, n2), axes=(0, 1, 2))  # includes the 1/N
    return np.asarray(v_diag) * np.asarray(x) + back.reshape(-1)


def dpp_sites(waters_angstrom):
    """Rigid-water DPP site tables (sites, charges, charge_site, dipoles, dipole_site, iters)."""
    w = np.ascontiguousarray(waters_angstrom, dtype=np.float64).reshape(-1)
    nw = len(w) // 9
    sites = np.empty(12 * nw)
    q = np.empty(3 * nw)
    qs = np.empty(3 * nw, dtype=np.int32)
    d = np.empty(9 * nw)
    ds = np.empty(3 * nw, dtype=np.int32)
    it = lib().or_dpp_sites(nw, _d(w), _d(sites), _d(q), _i(qs), _d(d), _i(ds))
    return sites, q, qs, d, ds, it


def scpol_inva(pos, alpha, a_thole=0.3):
    """A = (alpha^-1 - T)^-1 (or_scpol_inva), (3 npp, 3 npp)."""
    L = lib()
    L.or_scpol_inva.argtypes = [C.c_int, _dp, _dp, C.c_double, _dp]
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    a = np.empty((3 * len(alpha), 3 * len(alpha)))
    if L.or_scpol_inva(len(alpha), _d(pos), _d(alpha), float(a_thole), _d(a)) != 0:
        raise ValueError("singular polarisation matrix")
    return a


def hf_gradient_final(nsites, tmu, mcm, dT_x, dT_y, dT_z, dEfield, pol_grad, gradient):
    """gradient += FinalGradient terms - pol_grad (or_hf_gradient_final), in place."""
    L = lib()
    L.or_hf_gradient_final.argtypes = [C.c_int, C.c_int] + [_dp] * 8
    arr = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in (tmu, mcm, dT_x, dT_y, dT_z, dEfield)]
    pgd = None if pol_grad is None else np.ascontiguousarray(pol_grad, dtype=np.float64)
    L.or_hf_gradient_final(int(nsites), len(arr[0]) // 3, *[_d(a) for a in arr], _d(pgd) if pgd is not None else None,
                           _d(gradient))
    return gradient


def dual_extend(n, nc, wf_coarse):
    """Fine start vector from a coarse state (or_dual_extend); n, nc: points per axis."""
    L = lib()
    L.or_dual_extend.argtypes = [C.c_int, C.c_int, _dp, _dp]
    wc = np.ascontiguousarray(wf_coarse, dtype=np.float64)
    out = np.empty(n ** 3)
    L.or_dual_extend(int(n), int(nc), _d(wc), _d(out))
    return out


def small_to_large(n, xmin, dx, wf, N, XMIN, DX):
    """Small2Large (eight-point interpolation, normalised) onto the grid N, XMIN + I DX."""
    out = np.empty(int(np.prod(N)))
    L = lib()
    L.or_small_to_large.argtypes = [_ip, _dp, _dp, _dp, _ip, _dp, _dp, _dp]
    a = lambda v, t=np.float64: np.ascontiguousarray(v, dtype=t)
    L.or_small_to_large(_i(a(n, np.int32)), _d(a(xmin)), _d(a(dx)), _d(a(wf)), _i(a(N, np.int32)), _d(a(XMIN)),
                        _d(a(DX)), _d(out))
    return out


def syev(a):
    n = a.shape[0]
    A = np.asfortranarray(a, dtype=np.float64).copy()
    w = np.empty(n)
    V = np.empty((n, n), order="F")
    lib().or_syev(n, A.ctypes.data_as(_dp), n, _d(w), V.ctypes.data_as(_dp), n)
    return w, V


# ---------------------------------------------------------------- reference driver

def read_records(path):
    """Parse a record file written by the reference driver."""
    out = {}
    with open(path, "rb") as f:
        if f.read(8) != b"PGREC1\0\0":
            raise ValueError("not a record file")
        while True:
            head = f.read(64)
            if len(head) < 64:
                break
            name = head.split(b"\0", 1)[0].decode()
            kind = f.read(8)[:1]
            (n,) = struct.unpack("<Q", f.read(8))
            if kind == b"d":
                out[name] = np.frombuffer(f.read(8 * n), dtype="<f8").copy()
            else:
                out[name] = np.frombuffer(f.read(4 * n), dtype="<i4").copy()
    return out


def have_reference() -> bool:
    return os.path.exists(REF_BIN)


def run_reference(n, L, waters=None, ions=None, nstates=1, method=2, maxsub=20, maxiter=100, ptol=5, startvec=1,
                  spherical_k=None, matvec_seed=None, fulldiag=False, diagonalize=True, dump_wavefn=True,
                  threads=None, observables=None, poltype=None, gradient=False, dual=False, rtol=None, fft=False):
    """Run the reference CPU code (built by oracle/ref/Makefile) on one configuration.
    fft: the FFT kinetic path instead (DVRType 3 grid, KE_diag, two
    VectorFFT::apply products on seeded vectors; nothing else runs)."""
    if not have_reference():
        raise FileNotFoundError(REF_BIN)
    os.makedirs(os.path.join(HERE, "_ref", "tmp"), exist_ok=True)
    with tempfile.TemporaryDirectory(dir=os.path.join(HERE, "_ref", "tmp")) as td:
        inp = os.path.join(td, "in.txt")
        out = os.path.join(td, "out.rec")
        lines = [f"grid {n[0]} {n[1]} {n[2]} {L[0]!r} {L[1]!r} {L[2]!r}",
                 f"diag {nstates} {method} {maxsub} {maxiter} {ptol} {startvec}"]
        if waters is not None and len(waters):
            w = np.asarray(waters, dtype=np.float64).reshape(-1, 9)
            lines.append(f"waters {len(w)}")
            lines += [" ".join(repr(float(c)) for c in row) for row in w]
        if ions is not None and len(ions):
            io = np.asarray(ions, dtype=np.float64).reshape(-1, 4)
            lines.append(f"ions {len(io)}")
            lines += [" ".join(repr(float(c)) for c in row) for row in io]
        if spherical_k is not None:
            lines.append(f"spherical {spherical_k!r}")
        if matvec_seed is not None:
            lines.append(f"matvec_seed {int(matvec_seed)}")
        if observables is not None:
            lines.append("observables {} {} {}".format(*[int(v) for v in observables]))
        if poltype is not None:
            lines.append(f"poltype {int(poltype)}")
        if gradient:
            lines.append("gradient 1")
        if dual:
            lines.append("dual 1")
        if rtol is not None:
            lines.append(f"rtol {float(rtol)!r}")
        if fft:
            lines.append("fft 1")
        lines += [f"fulldiag {int(fulldiag)}", f"diagonalize {int(diagonalize)}",
                  f"dump_wavefn {int(dump_wavefn)}", f"out {out}"]
        with open(inp, "w") as f:
            f.write("\n".join(lines) + "\n")
        env = dict(os.environ)
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        subprocess.run([REF_BIN, inp], check=True, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, env=env)
        return read_records(out)
