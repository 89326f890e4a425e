"""pisces_gb300 -- Python front end of libpisces_gb300.so (the GB300 eigensolve path).

Thin ctypes layer over the C ABI declared in include/pisces_gb300.h.  Device
arrays are torch CUDA tensors (float64, contiguous); host arrays are numpy.
There is no CPU fallback: if the library is missing or no GPU is present the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpisces_gb300.so")

PG_OK, PG_BAD_ARG, PG_OOM, PG_NOT_CONVERGED, PG_DEVICE_TIMEOUT, PG_NUMERIC, PG_CUDA, PG_UNSUPPORTED = range(8)
PG_FP64, PG_MIXED = 0, 1
_STATUS = {0: "ok", 1: "bad argument", 2: "out of memory", 3: "not converged", 4: "device timeout", 5: "numeric",
           6: "cuda error", 7: "unsupported"}


class PiscesError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{_STATUS.get(status, status)}: {msg}")
        self.status = status


class NotConverged(PiscesError):
    pass


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p


class Sites(C.Structure):
    """pg_sites: the electron-site lists (host pointers)."""
    _fields_ = [("nsites", C.c_int), ("sites", _dp),
                ("ncharges", C.c_int), ("charges", _dp), ("charge_site", _ip),
                ("ndipoles", C.c_int), ("dipoles", _dp), ("dipole_site", _ip),
                ("nsto", C.c_int), ("sto", _dp), ("sto_site", _ip),
                ("npol", C.c_int), ("pol_alpha", _dp), ("pol_site", _ip),
                ("charge_damp", C.c_double), ("dipole_damp", C.c_double), ("pol_damp", C.c_double)]


class ScPolModel(C.Structure):
    """pg_scpol_model: the self-consistent polarisation model (host pointers)."""
    _fields_ = [("npp", C.c_int), ("pol_site", _ip), ("inva", _dp), ("epc", _dp), ("damp_type", C.c_int),
                ("damp", C.c_double), ("vpol_ww", C.c_double)]


class SolveParams(C.Structure):
    _fields_ = [("nroots", C.c_int), ("maxsub", C.c_int), ("maxiter", C.c_int), ("ptol", C.c_int),
                ("corrflag", C.c_int), ("precision", C.c_int), ("startvec", C.c_int), ("refine", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("nconv", C.c_int), ("n_matvec", C.c_int), ("n_iter", C.c_int), ("n_restart", C.c_int),
                ("residual", C.c_double * 64), ("seconds", C.c_double), ("host_eig_seconds", C.c_double),
                ("device_wait_seconds", C.c_double)]

    def as_dict(self, nroots):
        return {"nconv": self.nconv, "n_matvec": self.n_matvec, "n_iter": self.n_iter, "n_restart": self.n_restart,
                "residual": list(self.residual[:nroots]), "seconds": self.seconds,
                "host_eig_seconds": self.host_eig_seconds, "device_wait_seconds": self.device_wait_seconds}


class Moments(C.Structure):
    """pg_moments: sum psi^2, <x,y,z>, <r^2> and the transition dipole with state 0."""
    _fields_ = [("norm", C.c_double), ("r", C.c_double * 3), ("r2", C.c_double), ("trans_dipole", C.c_double * 3)]


class EngineConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("slots", C.c_int), ("memory_budget", C.c_double),
                ("batch_matvecs", C.c_int), ("batch_window_us", C.c_int), ("warm_start", C.c_int)]


class Request(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("L", C.c_double * 3), ("nw", C.c_int), ("waters", _dp),
                ("nions", C.c_int), ("ions", _dp), ("params", SolveParams), ("key", C.c_long),
                ("evecs_host", _dp)]


class Result(C.Structure):
    _fields_ = [("id", C.c_long), ("status", C.c_int), ("nroots", C.c_int), ("warm_started", C.c_int),
                ("evals", C.c_double * 64), ("stats", SolveStats), ("queue_seconds", C.c_double),
                ("latency_seconds", C.c_double), ("error", C.c_char * 256)]


class EngineStats(C.Structure):
    _fields_ = [("submitted", C.c_long), ("completed", C.c_long), ("failed", C.c_long),
                ("warm_starts", C.c_long), ("batches", C.c_long), ("batched_products", C.c_long),
                ("peak_in_flight", C.c_int), ("peak_bytes", C.c_double)]


_lib = None

# exported C-ABI symbols (also checked by the CPU tests against the header)
SYMBOLS = {
    "pg_last_error": (C.c_char_p, []),
    "pg_version": (C.c_int, []),
    "pg_kernel_launches": (C.c_long, []),
    "pg_device_allocations": (C.c_long, []),
    "pg_sine_dvr": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, _dp, _dp, C.c_int]),
    "pg_grid_create": (C.c_int, [_ip, _dp, C.POINTER(_vp)]),
    "pg_grid_create_dvr": (C.c_int, [_ip, _dp, C.c_int, C.POINTER(_vp)]),
    "pg_fft_kinetic": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp]),
    "pg_grid_destroy": (C.c_int, [_vp]),
    "pg_grid_npoints": (C.c_long, [_vp]),
    "pg_grid_points": (C.c_int, [_vp, _dp, _dp, _dp]),
    "pg_grid_kinetic": (C.c_int, [_vp, C.c_int, _dp]),
    "pg_diagonal": (C.c_int, [_vp, _vp, _vp, _vp]),
    "pg_piab_start": (C.c_int, [_vp, _vp, _vp]),
    "pg_potential_eval": (C.c_int, [_vp, C.POINTER(Sites), _vp, _vp, _vp]),
    "pg_potential_ions_add": (C.c_int, [_vp, C.c_int, _dp, _dp, C.c_double, C.c_double, _vp, _vp]),
    "pg_potential_spherical": (C.c_int, [_vp, C.c_double, _vp, _vp]),
    "pg_water_sites": (C.c_int, [C.c_int, _dp, _dp, _dp, _ip, _dp, _ip, _ip]),
    "pg_water_default_tables": (C.c_int, [C.c_int, _dp, _dp, _ip, _dp, _ip, _dp, _ip, _dp, _ip, C.POINTER(Sites)]),
    "pg_hx": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, _vp]),
    "pg_hx_async": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, _vp]),
    "pg_grid_check": (C.c_int, [_vp, _vp]),
    "pg_grid_set_hx_kernel": (C.c_int, [_vp, C.c_int]),
    "pg_grid_hx_plan": (C.c_int, [_vp, C.c_char_p, C.c_int]),
    "pg_grid_hx_plan_for": (C.c_int, [_vp, C.c_int, C.c_char_p, C.c_int]),
    "pg_grid_set_hx_params": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int]),
    "pg_kinetic_precondition": (C.c_int, [_vp, _vp, C.c_int, _dp, C.c_int, _vp]),
    "pg_grid_set_precond_kernel": (C.c_int, [_vp, C.c_int]),
    "pg_grid_precond_plan": (C.c_int, [_vp, C.c_char_p, C.c_int]),
    "pg_davidson_create": (C.c_int, [C.POINTER(_vp)]),
    "pg_davidson_destroy": (C.c_int, [_vp]),
    "pg_davidson_work_size": (C.c_long, [C.c_int, C.c_int, C.c_int, C.c_int]),
    "pg_subspace_lowest": (C.c_int, [C.c_int, _dp, C.c_int, C.c_int, _dp, _dp, C.c_int]),
    "pg_davidson_set_preconditioner": (C.c_int, [_vp, _vp, C.c_int]),
    "pg_davidson_set_arithmetic": (C.c_int, [_vp, C.c_int]),
    "pg_davidson_rci": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _ip, _vp, _vp,
                                  _vp, _vp, _ip, _ip, _vp]),
    "pg_solve": (C.c_int, [_vp, _vp, C.POINTER(SolveParams), _dp, _vp, C.POINTER(SolveStats), _vp]),
    "pg_cluster_solve": (C.c_int, [_ip, _dp, C.c_int, _dp, C.c_int, _dp, C.POINTER(SolveParams), _dp, _dp,
                                   C.POINTER(SolveStats), _vp]),
    "pg_glibc_rand_check": (C.c_int, [C.c_int, _ip]),
    "pg_block_gram": (C.c_int, [C.c_long, _vp, C.c_int, _vp, C.c_int, _vp, C.c_int, _vp]),
    "pg_block_combine": (C.c_int, [C.c_long, _vp, C.c_int, _vp, C.c_int, _vp, C.c_int, _vp]),
    "pg_block_gram_noalloc": (C.c_int, [C.c_long, _vp, C.c_int, _vp, C.c_int, _vp, C.c_int, _vp]),
    "pg_split_twin": (C.c_int, [C.c_long, _vp, _vp, _vp]),
    "pg_water_scpol": (C.c_int, [C.c_int, _dp, _ip, _dp, _dp, _dp]),
    "pg_scpol_inva": (C.c_int, [C.c_int, _dp, _dp, C.c_double, _dp]),
    "pg_potential_scpol_add": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "pg_hf_gradient_grid": (C.c_int, [_vp, _vp, _vp, _vp, _dp, _dp, _dp, _vp]),
    "pg_hf_gradient_final": (C.c_int, [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "pg_dual_grid_coarse": (C.c_int, [_ip, _dp, _ip, _dp, _ip]),
    "pg_dual_grid_potential": (C.c_int, [_vp, _ip, _vp, _vp, _vp, C.c_double, _vp, C.POINTER(C.c_long), _vp]),
    "pg_dual_grid_extend": (C.c_int, [_vp, _ip, _vp, _vp, _vp]),
    "pg_block_gram_twin": (C.c_int, [C.c_long, _vp, C.c_int, _vp, C.c_int, _vp, _vp]),
    "pg_block_combine_twin": (C.c_int, [C.c_long, _vp, C.c_int, _vp, C.c_int, _vp, _vp, _vp]),
    "pg_expectation_values": (C.c_int, [_vp, _vp, C.c_int, C.POINTER(Moments), _vp]),
    "pg_energy_partition": (C.c_int, [_vp, _vp, C.c_int, _vp, _dp, _vp]),
    "pg_state_cube": (C.c_int, [_vp, _dp, _dp]),
    "pg_write_state_cube": (C.c_int, [_vp, _dp, C.c_int, C.c_char_p, C.c_int, _ip, _dp, C.c_int, _dp]),
    "pg_write_cube": (C.c_int, [C.c_char_p, C.c_int, _ip, _dp, _ip, _dp, _dp, _dp]),
    "pg_read_cube": (C.c_int, [C.c_char_p, _ip, _dp, _dp, _ip, _dp, C.c_long]),
    "pg_small_to_large": (C.c_int, [_ip, _dp, _dp, _dp, _vp, _vp, _vp]),
    "pg_request_footprint": (C.c_double, [C.POINTER(Request)]),
    "pg_engine_create": (C.c_int, [C.POINTER(EngineConfig), C.POINTER(_vp)]),
    "pg_engine_submit": (C.c_int, [_vp, C.POINTER(Request), C.POINTER(C.c_long)]),
    "pg_engine_wait": (C.c_int, [_vp, C.c_long, C.POINTER(Result), C.c_double]),
    "pg_engine_poll": (C.c_int, [_vp, C.POINTER(Result), C.c_int, _ip]),
    "pg_engine_get_stats": (C.c_int, [_vp, C.POINTER(EngineStats)]),
    "pg_engine_destroy": (C.c_int, [_vp]),
}


def lib():
    """Load libpisces_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PiscesError(PG_UNSUPPORTED, f"{LIB_PATH} is missing: build it with pisces-1_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SYMBOLS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status):
    if status != PG_OK:
        msg = lib().pg_last_error().decode(errors="replace")
        if status == PG_NOT_CONVERGED:
            raise NotConverged(status, msg)
        raise PiscesError(status, msg)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _dev(t):
    """Device pointer of a contiguous float64 CUDA tensor."""
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
        raise TypeError("expected a contiguous float64 CUDA tensor")
    return C.c_void_p(t.data_ptr())


def _stream(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return C.c_void_p(int(stream))


def fft_kinetic(n, L, mu=1.0):
    """Periodic FFT kinetic term on (-L/2, L/2): grid points, plane-wave
    energies and the n x n circulant matrix of the per-axis operator."""
    x, e, t = np.empty(n), np.empty(n), np.empty(n * n)
    _check(lib().pg_fft_kinetic(n, mu, -0.5 * L, 0.5 * L, _d(x), _d(e), _d(t)))
    return x, e, t.reshape(n, n)


def sine_dvr(n, L, mu=1.0, packed=True):
    """1-D sine DVR on (-L/2, L/2): grid points and kinetic matrix (packed or full)."""
    x = np.empty(n)
    t = np.empty(n * (n + 1) // 2 if packed else n * n)
    _check(lib().pg_sine_dvr(n, mu, -0.5 * L, 0.5 * L, _d(x), _d(t), 0 if packed else n))
    return x, (t if packed else t.reshape(n, n))


class WaterTables:
    """Default electron-water model tables built from water coordinates (Angstrom)."""

    def __init__(self, waters_angstrom):
        w = np.ascontiguousarray(waters_angstrom, dtype=np.float64).reshape(-1)
        nw = len(w) // 9
        if nw * 9 != len(w) or nw == 0:
            raise ValueError("waters must be n x 9 Angstrom coordinates")
        self.nw = nw
        self.waters = w
        self.sites = np.empty(12 * nw)
        self.charges = np.empty(3 * nw)
        self.charge_site = np.empty(3 * nw, dtype=np.int32)
        self.dipoles = np.empty(9 * nw)
        self.dipole_site = np.empty(3 * nw, dtype=np.int32)
        it = C.c_int(0)
        _check(lib().pg_water_sites(nw, _d(w), _d(self.sites), _d(self.charges), _i(self.charge_site),
                                    _d(self.dipoles), _i(self.dipole_site), C.byref(it)))
        self.scf_iters = it.value
        self.sto = np.empty(8 * nw)
        self.sto_site = np.empty(4 * nw, dtype=np.int32)
        self.pol_alpha = np.empty(nw)
        self.pol_site = np.empty(nw, dtype=np.int32)
        self.table = Sites()
        _check(lib().pg_water_default_tables(nw, _d(self.sites), _d(self.charges), _i(self.charge_site),
                                             _d(self.dipoles), _i(self.dipole_site), _d(self.sto), _i(self.sto_site),
                                             _d(self.pol_alpha), _i(self.pol_site), C.byref(self.table)))

    @classmethod
    def from_lists(cls, sites, charges, charge_site, dipoles, dipole_site):
        """Tables from site lists produced elsewhere (e.g. by the reference)."""
        self = cls.__new__(cls)
        self.sites = np.ascontiguousarray(sites, dtype=np.float64)
        nw = len(self.sites) // 12
        self.nw = nw
        self.charges = np.ascontiguousarray(charges, dtype=np.float64)
        self.charge_site = np.ascontiguousarray(charge_site, dtype=np.int32)
        self.dipoles = np.ascontiguousarray(dipoles, dtype=np.float64)
        self.dipole_site = np.ascontiguousarray(dipole_site, dtype=np.int32)
        self.scf_iters = None
        self.sto = np.empty(8 * nw)
        self.sto_site = np.empty(4 * nw, dtype=np.int32)
        self.pol_alpha = np.empty(nw)
        self.pol_site = np.empty(nw, dtype=np.int32)
        self.table = Sites()
        _check(lib().pg_water_default_tables(nw, _d(self.sites), _d(self.charges), _i(self.charge_site),
                                             _d(self.dipoles), _i(self.dipole_site), _d(self.sto), _i(self.sto_site),
                                             _d(self.pol_alpha), _i(self.pol_site), C.byref(self.table)))
        return self


def dual_grid_coarse(n, L):
    """(nc, Lc, spacing) of the dual grid's coarse grid (pg_dual_grid_coarse)."""
    n = np.ascontiguousarray(np.broadcast_to(n, 3), dtype=np.int32)
    L = np.ascontiguousarray(np.broadcast_to(L, 3), dtype=np.float64)
    nc, Lc, sp = np.empty(3, dtype=np.int32), np.empty(3), C.c_int(0)
    _check(lib().pg_dual_grid_coarse(_i(n), _d(L), _i(nc), _d(Lc), C.byref(sp)))
    return tuple(int(v) for v in nc), tuple(float(v) for v in Lc), sp.value


def scpol_inva(pos_bohr, alpha, a_thole=0.3):
    """A = (alpha^-1 - T)^-1 of point-polarisable atoms (pg_scpol_inva), (3 npp, 3 npp)."""
    pos = np.ascontiguousarray(pos_bohr, dtype=np.float64).reshape(-1)
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    npp = len(alpha)
    if len(pos) != 3 * npp:
        raise ValueError("pos must hold 3 coordinates per polarisable atom")
    a = np.empty((3 * npp, 3 * npp))
    _check(lib().pg_scpol_inva(npp, _d(pos), _d(alpha), float(a_thole), _d(a)))
    return a


class ScPol:
    """The self-consistent polarisation model of a water cluster (PolType 3/5/6
    of the reference): polarisable atoms O, H1, H2 of every water, A, Epc and
    the water-water offset; `tables` are the electron's charge and
    repulsive-core lists of the same cluster, without induced dipoles or the
    one-site polarisation term."""

    def __init__(self, waters_angstrom=None, damp=2.536, damp_type=2, a_thole=0.3, tables=None, pol_site=None,
                 inva=None, epc=None, vpol_ww=None):
        if waters_angstrom is not None:
            w = WaterTables(waters_angstrom)
            nw = w.nw
            ps = np.empty(3 * nw, dtype=np.int32)
            alpha = np.empty(3 * nw)
            epc_ = np.empty(9 * nw)
            vww = C.c_double(0)
            _check(lib().pg_water_scpol(nw, _d(w.waters), _i(ps), _d(alpha), _d(epc_), C.byref(vww)))
            pos = w.sites.reshape(-1, 3)[ps]
            self.base = w
            self.alpha = alpha
            pol_site, epc, vpol_ww = ps, epc_, vww.value
            inva = scpol_inva(pos, alpha, a_thole) if inva is None else inva
            tables = w
        self.base = tables
        self.pol_site = np.ascontiguousarray(pol_site, dtype=np.int32)
        self.inva = np.ascontiguousarray(inva, dtype=np.float64)
        self.epc = np.ascontiguousarray(epc, dtype=np.float64).reshape(-1)
        self.vpol_ww = float(vpol_ww)
        npp = len(self.pol_site)
        if self.inva.size != 9 * npp * npp or self.epc.size != 3 * npp:
            raise ValueError("inva must be (3 npp)^2 and epc 3 npp values")
        self.model = ScPolModel(npp, _i(self.pol_site), _d(self.inva), _d(self.epc), int(damp_type), float(damp),
                                self.vpol_ww)
        # the charges and Slater cores of the cluster, no dipoles, no
        # one-site polarisation
        t = tables.table
        self.table = Sites(t.nsites, t.sites, t.ncharges, t.charges, t.charge_site, 0, None, None, t.nsto, t.sto,
                           t.sto_site, 0, None, None, t.charge_damp, t.dipole_damp, t.pol_damp)


class Grid:
    """3-D grid on the current CUDA device (pg_grid): dvrtype 2 = sine DVR,
    3 = periodic FFT kinetic term (the reference's DVRType values)."""

    def __init__(self, n, L, dvrtype=2):
        n = np.ascontiguousarray(np.broadcast_to(n, 3), dtype=np.int32)
        L = np.ascontiguousarray(np.broadcast_to(L, 3), dtype=np.float64)
        h = _vp()
        _check(lib().pg_grid_create_dvr(_i(n), _d(L), int(dvrtype), C.byref(h)))
        self.dvrtype = int(dvrtype)
        self._h = h
        self.n = tuple(int(v) for v in n)
        self.L = tuple(float(v) for v in L)
        self.N = int(lib().pg_grid_npoints(h))

    def close(self):
        if self._h:
            lib().pg_grid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def points(self):
        xs = [np.empty(m) for m in self.n]
        _check(lib().pg_grid_points(self._h, _d(xs[0]), _d(xs[1]), _d(xs[2])))
        return xs

    def kinetic(self, axis):
        t = np.empty((self.n[axis], self.n[axis]))
        _check(lib().pg_grid_kinetic(self._h, axis, _d(t)))
        return t

    def _new(self, count=1):
        import torch
        return torch.empty(count * self.N, dtype=torch.float64, device="cuda")

    def potential(self, tables: WaterTables, parts=False, stream=None):
        v = self._new()
        p = self._new(4) if parts else None
        _check(lib().pg_potential_eval(self._h, C.byref(tables.table), _dev(v), _dev(p) if parts else None,
                                       _stream(stream)))
        return (v, p.view(4, self.N)) if parts else v

    def potential_scpol(self, model: ScPol, parts=False, stream=None):
        """V(r) of the self-consistent polarisation model: charges and
        repulsive core (pg_potential_eval) plus the polarisation term
        (pg_potential_scpol_add)."""
        v = self._new()
        p = self._new(4) if parts else None
        _check(lib().pg_potential_eval(self._h, C.byref(model.table), _dev(v), _dev(p) if parts else None,
                                       _stream(stream)))
        _check(lib().pg_potential_scpol_add(self._h, C.byref(model.table), C.byref(model.model), _dev(v),
                                            _dev(p) if parts else None, _stream(stream)))
        return (v, p.view(4, self.N)) if parts else v

    def scpol_add(self, model: ScPol, v, parts=None, stream=None):
        """v += the self-consistent polarisation term (pg_potential_scpol_add)."""
        _check(lib().pg_potential_scpol_add(self._h, C.byref(model.table), C.byref(model.model), _dev(v),
                                            _dev(parts) if parts is not None else None, _stream(stream)))
        return v

    def dual_potential(self, nc, v_coarse, model: ScPol, rtol, stream=None):
        """(V, exact point count) of PolType 6 from the coarse grid's V (pg_dual_grid_potential)."""
        nc = np.ascontiguousarray(np.broadcast_to(nc, 3), dtype=np.int32)
        v = self._new()
        ne = C.c_long(0)
        _check(lib().pg_dual_grid_potential(self._h, _i(nc), _dev(v_coarse), C.byref(model.table),
                                            C.byref(model.model), float(rtol), _dev(v), C.byref(ne), _stream(stream)))
        return v, ne.value

    def dual_extend(self, nc, wf_coarse, stream=None):
        """Fine-grid start vector from a coarse state (pg_dual_grid_extend)."""
        nc = np.ascontiguousarray(np.broadcast_to(nc, 3), dtype=np.int32)
        w = self._new()
        _check(lib().pg_dual_grid_extend(self._h, _i(nc), _dev(wf_coarse), _dev(w), _stream(stream)))
        return w

    def hf_gradient_grid(self, model: ScPol, psi, stream=None):
        """(grad[3 nsites], tmu[3 npp], mcm[3 npp, 3 npp]): the grid sums of the
        electron's Hellmann-Feynman gradient for the density psi^2
        (pg_hf_gradient_grid)."""
        ns = model.table.nsites
        n = 3 * len(model.pol_site)
        grad, tmu, mcm = np.empty(3 * ns), np.empty(n), np.empty((n, n))
        _check(lib().pg_hf_gradient_grid(self._h, C.byref(model.table), C.byref(model.model), _dev(psi),
                                         _d(grad), _d(tmu), _d(mcm), _stream(stream)))
        return grad, tmu, mcm

    def add_ions(self, v, pos_bohr, q, r_cation=2.9, r_anion=1.0, stream=None):
        pos = np.ascontiguousarray(pos_bohr, dtype=np.float64).reshape(-1)
        q = np.ascontiguousarray(q, dtype=np.float64)
        _check(lib().pg_potential_ions_add(self._h, len(q), _d(pos), _d(q), r_cation, r_anion, _dev(v),
                                           _stream(stream)))
        return v

    def spherical(self, k, stream=None):
        v = self._new()
        _check(lib().pg_potential_spherical(self._h, float(k), _dev(v), _stream(stream)))
        return v

    def diagonal(self, v, stream=None):
        d = self._new()
        _check(lib().pg_diagonal(self._h, _dev(v), _dev(d), _stream(stream)))
        return d

    def piab(self, stream=None):
        w = self._new()
        _check(lib().pg_piab_start(self._h, _dev(w), _stream(stream)))
        return w

    def hx(self, v, X, nvec=None, precision=PG_FP64, out=None, stream=None, wait=True):
        """Y = H X.  wait=False: queue only (pg_hx_async); call check() later."""
        nvec = X.numel() // self.N if nvec is None else nvec
        Y = self._new(nvec) if out is None else out
        fn = lib().pg_hx if wait else lib().pg_hx_async
        _check(fn(self._h, _dev(v), _dev(X), _dev(Y), nvec, precision, _stream(stream)))
        return Y

    def set_hx_kernel(self, kind):
        """Mixed H*X kernel of this grid: 0 automatic, 1 three axis passes, 2 fused."""
        _check(lib().pg_grid_set_hx_kernel(self._h, int(kind)))

    def set_hx_params(self, kind=0, lag=0, ctas=0, form=0):
        """Override the tuned mixed H*X launch parameters (pg_grid_set_hx_params; 0 = tuned)."""
        _check(lib().pg_grid_set_hx_params(self._h, int(kind), int(lag), int(ctas), int(form)))

    def hx_plan(self, nvec=1):
        """One-line description of the mixed H*X kernel this grid uses for nvec vectors."""
        buf = C.create_string_buffer(512)
        _check(lib().pg_grid_hx_plan_for(self._h, int(nvec), buf, 512))
        return buf.value.decode()

    def precondition(self, R, sigma, precision=PG_MIXED, stream=None):
        """R <- (T - sigma_j)^-1 R in place for the len(sigma) vectors of R (pg_kinetic_precondition)."""
        sg = np.ascontiguousarray(np.atleast_1d(np.asarray(sigma, dtype=np.float64)))
        _check(lib().pg_kinetic_precondition(self._h, _dev(R), len(sg), sg.ctypes.data_as(_dp), precision,
                                             _stream(stream)))
        return R

    def set_precond_kernel(self, kind):
        """Mixed-form preconditioner kernel of this grid: 0 automatic (FP16 kernel), 1 axis passes."""
        _check(lib().pg_grid_set_precond_kernel(self._h, int(kind)))

    def precond_plan(self):
        """One-line description of the mixed-form preconditioner this grid uses."""
        buf = C.create_string_buffer(512)
        _check(lib().pg_grid_precond_plan(self._h, buf, 512))
        return buf.value.decode()

    def check(self, stream=None):
        """Waits for the stream and reports a tensor-core wait timeout (pg_grid_check)."""
        _check(lib().pg_grid_check(self._h, _stream(stream)))

    def solve(self, v, nroots=1, maxsub=20, maxiter=100, ptol=5, corrflag=1, precision=PG_FP64, startvec=1,
              refine=1, start=None, stream=None, raise_on_nonconv=True):
        """Device Davidson eigensolve; returns (evals, evecs[nroots, N] on the device, stats dict)."""
        import torch
        if start is not None and startvec != 3:
            startvec = 0
        p = SolveParams(nroots, maxsub, maxiter, ptol, corrflag, precision, startvec, refine)
        ev = np.zeros(nroots)
        vec = torch.empty(nroots * self.N, dtype=torch.float64, device="cuda")
        if start is not None:
            # startvec 3: only the first column is given
            vec[:start.numel()].copy_(start.reshape(-1))
        st = SolveStats()
        s = lib().pg_solve(self._h, _dev(v), C.byref(p), _d(ev), _dev(vec), C.byref(st), _stream(stream))
        if s != PG_OK and (s != PG_NOT_CONVERGED or raise_on_nonconv):
            _check(s)
        return ev, vec.view(nroots, self.N), st.as_dict(nroots)


    # ------------------------------------------------ observables and cube files

    def expectation_values(self, vecs, nstates=None, stream=None):
        """pg_expectation_values: list of dicts (norm, r, r2, trans_dipole) per state."""
        nstates = vecs.numel() // self.N if nstates is None else nstates
        out = (Moments * nstates)()
        _check(lib().pg_expectation_values(self._h, _dev(vecs), nstates, out, _stream(stream)))
        return [{"norm": m.norm, "r": list(m.r), "r2": m.r2, "trans_dipole": list(m.trans_dipole)} for m in out]

    def energy_partition(self, vecs, parts, nstates=None, stream=None):
        """pg_energy_partition: [nstates, 4] sums of psi^2 times the potential parts (hartree)."""
        nstates = vecs.numel() // self.N if nstates is None else nstates
        out = np.empty(4 * nstates)
        _check(lib().pg_energy_partition(self._h, _dev(vecs), nstates, _dev(parts), _d(out), _stream(stream)))
        return out.reshape(nstates, 4)

    def state_cube(self, wf_host):
        """pg_state_cube: a state's values in cube order, in bohr^-3/2."""
        wf = np.ascontiguousarray(wf_host, dtype=np.float64)
        out = np.empty(self.N)
        _check(lib().pg_state_cube(self._h, _d(wf), _d(out)))
        return out

    def write_state_cube(self, path, wf_host, iwf=1, Z=(), pos_angstrom=(), cubeflag=0):
        """pg_write_state_cube; returns sum rho^2 dV."""
        wf = np.ascontiguousarray(wf_host, dtype=np.float64)
        Zs = np.ascontiguousarray(Z, dtype=np.int32)
        pos = np.ascontiguousarray(pos_angstrom, dtype=np.float64).reshape(-1)
        integral = C.c_double(0)
        _check(lib().pg_write_state_cube(self._h, _d(wf), int(iwf), os.fsencode(path), len(Zs),
                                         _i(Zs) if len(Zs) else None, _d(pos) if len(Zs) else None, int(cubeflag),
                                         C.byref(integral)))
        return integral.value

    def small_to_large(self, n, xmin, dx, wf_small, stream=None):
        """pg_small_to_large: a start vector on this grid from a smaller grid's values (cube order)."""
        out = self._new()
        n = np.ascontiguousarray(n, dtype=np.int32)
        xmin = np.ascontiguousarray(xmin, dtype=np.float64)
        dx = np.ascontiguousarray(dx, dtype=np.float64)
        wf = np.ascontiguousarray(wf_small, dtype=np.float64)
        _check(lib().pg_small_to_large(_i(n), _d(xmin), _d(dx), _d(wf), self._h, _dev(out), _stream(stream)))
        return out


def write_cube(path, npts, x0, dx, cube, Z=(), pos_angstrom=()):
    """pg_write_cube: a Gaussian cube of any grid function (values with z fastest)."""
    npts = np.ascontiguousarray(npts, dtype=np.int32)
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    dx = np.ascontiguousarray(dx, dtype=np.float64)
    cube = np.ascontiguousarray(cube, dtype=np.float64)
    Zs = np.ascontiguousarray(Z, dtype=np.int32)
    pos = np.ascontiguousarray(pos_angstrom, dtype=np.float64).reshape(-1)
    _check(lib().pg_write_cube(os.fsencode(path), len(Zs), _i(Zs) if len(Zs) else None,
                               _d(pos) if len(Zs) else None, _i(npts), _d(x0), _d(dx), _d(cube)))


def read_cube(path):
    """pg_read_cube: (npts, x0, dx, natoms, values with z fastest)."""
    npts = np.zeros(3, dtype=np.int32)
    x0, dx = np.zeros(3), np.zeros(3)
    nat = C.c_int(0)
    _check(lib().pg_read_cube(os.fsencode(path), _i(npts), _d(x0), _d(dx), C.byref(nat), None, 0))
    cube = np.empty(int(np.prod(npts)))
    _check(lib().pg_read_cube(os.fsencode(path), _i(npts), _d(x0), _d(dx), C.byref(nat), _d(cube), len(cube)))
    return npts, x0, dx, nat.value, cube


class Davidson:
    """Reverse-communication Davidson (pg_davidson_rci), the drop-in for the
    reference's Davidson() with a caller-owned state instead of statics."""

    def __init__(self):
        h = _vp()
        _check(lib().pg_davidson_create(C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            lib().pg_davidson_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def work_size(ndim, maxsub, nroots, corrflag):
        return int(lib().pg_davidson_work_size(ndim, maxsub, nroots, corrflag))

    def set_arithmetic(self, precision):
        """Subspace arithmetic of this handle (pg_davidson_set_arithmetic), set before a solve."""
        _check(lib().pg_davidson_set_arithmetic(self._h, precision))

    def step(self, ndim, maxsub, nroots, maxmacro, tol, corrflag, evals, nconv, B, Z, diag, work, inout,
             stream=None):
        """One call: returns (status, ret) with ret as the reference's return code."""
        ret = C.c_int(0)
        s = lib().pg_davidson_rci(self._h, ndim, maxsub, nroots, maxmacro, tol, corrflag, _d(evals), C.byref(nconv),
                                  _dev(B), _dev(Z), _dev(diag), _dev(work), _i(inout), C.byref(ret), _stream(stream))
        return s, ret.value


def cluster_solve(n, L, waters_angstrom, ions=None, nroots=1, maxsub=20, maxiter=100, ptol=5, corrflag=1,
                  precision=PG_FP64, startvec=1, refine=1, want_vectors=True, stream=None):
    """Whole single point from host data (pg_cluster_solve): eigenvalues (and vectors) on the host."""
    n = np.ascontiguousarray(n, dtype=np.int32)
    L = np.ascontiguousarray(L, dtype=np.float64)
    w = np.ascontiguousarray(waters_angstrom, dtype=np.float64).reshape(-1)
    io = np.ascontiguousarray(ions if ions is not None else np.zeros((0, 4)), dtype=np.float64).reshape(-1)
    N = int(np.prod(n))
    ev = np.zeros(nroots)
    vec = np.empty(nroots * N) if want_vectors else None
    p = SolveParams(nroots, maxsub, maxiter, ptol, corrflag, precision, startvec, refine)
    st = SolveStats()
    s = lib().pg_cluster_solve(_i(n), _d(L), len(w) // 9, _d(w), len(io) // 4, _d(io) if len(io) else None,
                               C.byref(p), _d(ev), _d(vec) if want_vectors else None, C.byref(st),
                               _stream(stream) if stream is not None else None)
    _check(s)
    return ev, (vec.reshape(nroots, N) if want_vectors else None), st.as_dict(nroots)


def dual_single_point(n, L, model: ScPol, rtol=20.0, nroots=1, maxsub=20, maxiter=100, ptol=5, corrflag=1,
                      precision=PG_FP64, refine=1, stream=None):
    """The dual-grid single point (PotFlag[3] = 6 of
    ClusterAnion::EnergyFromConfiguration, src/ClusterAnion.cpp:211-290):
    the self-consistent model (PolType 3) solved on the coarse grid of
    pg_dual_grid_coarse, V of PolType 6 on the n^3 grid from the coarse V
    (pg_dual_grid_potential), then the fine solve from the coarse ground
    state interpolated onto it (pg_dual_grid_extend; startvec 3).
    Returns a dict: evals, evecs (device), v (device), n_exact, stats, and
    the coarse grid's nc, Lc, evals."""
    nc, Lc, _ = dual_grid_coarse(n, L)
    coarse = Grid(nc, Lc)
    vc = coarse.potential_scpol(model, stream=stream)
    kw = dict(maxsub=maxsub, maxiter=maxiter, ptol=ptol, corrflag=corrflag, precision=precision, refine=refine,
              stream=stream)
    ec, wc, _ = coarse.solve(vc, nroots=nroots, startvec=1, **kw)
    fine = Grid(np.broadcast_to(n, 3), np.broadcast_to(L, 3))
    v, n_exact = fine.dual_potential(nc, vc, model, rtol, stream=stream)
    start = fine.dual_extend(nc, wc[0], stream=stream)
    ev, vec, st = fine.solve(v, nroots=nroots, startvec=3, start=start, **kw)
    return {"evals": ev, "evecs": vec, "v": v, "n_exact": n_exact, "stats": st, "grid": fine, "coarse_n": nc,
            "coarse_L": Lc, "coarse_evals": ec}


def _check_block_args(P, Q, out, nout):
    """P and Q are 2-D blocks of equal length on one device; out holds nout values there."""
    if P.dim() != 2 or Q.dim() != 2 or P.shape[1] != Q.shape[1]:
        raise ValueError(f"blocks must be 2-D with equal rows, got {tuple(P.shape)} and {tuple(Q.shape)}")
    if P.device != Q.device:
        raise ValueError(f"P is on {P.device}, Q on {Q.device}")
    if out is not None:
        if out.device != P.device:
            raise ValueError(f"out is on {out.device}, the blocks on {P.device}")
        if out.numel() < nout:
            raise ValueError(f"out holds {out.numel()} values, {nout} needed")


def block_gram(P, Q, precision=PG_FP64, out=None, stream=None):
    """out[a, b] = P_a . Q_b for torch CUDA float64 blocks P (np x n), Q (nq x n)."""
    import torch
    np_, n = P.shape
    nq = Q.shape[0]
    _check_block_args(P, Q, out, np_ * nq)
    if out is None:
        out = torch.empty(np_ * nq, dtype=torch.float64, device=P.device)
    _check(lib().pg_block_gram(n, _dev(P), np_, _dev(Q), nq, _dev(out), precision, _stream(stream)))
    return out.view(-1)[:np_ * nq].view(np_, nq)


def block_gram_noalloc(P, Q, out, precision=PG_FP64, stream=None):
    """block_gram through pg_block_gram_noalloc: the library allocates nothing
    (out must be given; np * nq <= 256)."""
    np_, n = P.shape
    nq = Q.shape[0]
    _check_block_args(P, Q, out, np_ * nq)
    _check(lib().pg_block_gram_noalloc(n, _dev(P), np_, _dev(Q), nq, _dev(out), precision, _stream(stream)))
    return out.view(-1)[:np_ * nq].view(np_, nq)


def hf_gradient_final(nsites, tmu, mcm, dT_x, dT_y, dT_z, dEfield, pol_grad, gradient):
    """gradient += the FinalGradient terms - pol_grad (pg_hf_gradient_final), in place."""
    tmu = np.ascontiguousarray(tmu, dtype=np.float64)
    npp = len(tmu) // 3
    args = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in (mcm, dT_x, dT_y, dT_z, dEfield)]
    pg_ = None if pol_grad is None else np.ascontiguousarray(pol_grad, dtype=np.float64)
    if gradient.dtype != np.float64 or not gradient.flags.c_contiguous:
        raise TypeError("gradient must be a contiguous float64 array")
    _check(lib().pg_hf_gradient_final(int(nsites), npp, _d(tmu), *[_d(a) for a in args],
                                      _d(pg_) if pg_ is not None else None, _d(gradient)))
    return gradient


def split_twin(X, out=None, stream=None):
    """Double-float twins of a float64 CUDA tensor (pg_split_twin; same shape, float2 (hi, lo) per value)."""
    import torch
    out = torch.empty_like(X) if out is None else out
    _check(lib().pg_split_twin(X.numel(), _dev(X), _dev(out), _stream(stream)))
    return out


def block_gram_twin(Pt, Qt, out=None, stream=None):
    """out[a, b] = P_a . Q_b from twins (pg_block_gram_twin)."""
    import torch
    np_, n = Pt.shape
    nq = Qt.shape[0]
    _check_block_args(Pt, Qt, out, np_ * nq)
    if out is None:
        out = torch.empty(np_ * nq, dtype=torch.float64, device=Pt.device)
    _check(lib().pg_block_gram_twin(n, _dev(Pt), np_, _dev(Qt), nq, _dev(out), _stream(stream)))
    return out.view(-1)[:np_ * nq].view(np_, nq)


def block_combine_twin(Pt, Cm, out=None, out_twin=None, stream=None):
    """Y_r = sum_a P_a C[a, r] from twins of P (pg_block_combine_twin); out_twin receives Y's twins."""
    import torch
    np_, n = Pt.shape
    ny = Cm.shape[1]
    if out is None:
        out = torch.empty(ny, n, dtype=torch.float64, device=Pt.device)
    Cc = Cm.contiguous()
    _check(lib().pg_block_combine_twin(n, _dev(Pt), np_, _dev(Cc), ny, _dev(out),
                                       _dev(out_twin) if out_twin is not None else None, _stream(stream)))
    return out


def block_combine(P, Cm, precision=PG_FP64, out=None, stream=None):
    """Y_r = sum_a P_a C[a, r] for torch CUDA float64 P (np x n), C (np x ny)."""
    import torch
    np_, n = P.shape
    ny = Cm.shape[1]
    if out is None:
        out = torch.empty(ny, n, dtype=torch.float64, device=P.device)
    Cc = Cm.contiguous()
    _check(lib().pg_block_combine(n, _dev(P), np_, _dev(Cc), ny, _dev(out), precision, _stream(stream)))
    return out


def subspace_lowest(S, k):
    """k lowest eigenpairs of a symmetric matrix (upper triangle read) with the
    library's subspace eigensolver."""
    S = np.asfortranarray(S, dtype=np.float64)
    m = S.shape[0]
    w = np.empty(k)
    V = np.empty((m, k), order="F")
    _check(lib().pg_subspace_lowest(m, S.ctypes.data_as(_dp), m, k, _d(w), V.ctypes.data_as(_dp), m))
    return w, V


def glibc_rand_stream(count):
    """The library's restatement of the C library rand() sequence after srand(1)."""
    out = np.empty(count, dtype=np.int32)
    lib().pg_glibc_rand_check(count, _i(out))
    return out


def _result_dict(r: Result):
    nr = r.nroots
    return {"id": r.id, "status": r.status, "evals": list(r.evals[:nr]), "warm_started": bool(r.warm_started),
            "stats": r.stats.as_dict(nr), "queue_seconds": r.queue_seconds, "latency_seconds": r.latency_seconds,
            "error": r.error.decode(errors="replace")}


class Engine:
    """The serving engine (pg_engine_*): concurrent single points with
    footprint admission, warm start per key and merged mixed-form H*X."""

    def __init__(self, slots=8, memory_budget=0.0, batch_matvecs=True, batch_window_us=200, warm_start=True,
                 device=-1):
        self._h = _vp()
        self.config = EngineConfig(device, slots, memory_budget, int(batch_matvecs), batch_window_us,
                                   int(warm_start))
        _check(lib().pg_engine_create(C.byref(self.config), C.byref(self._h)))
        self._keep = {}  # host arrays that must live until their request is done

    def close(self):
        if self._h:
            lib().pg_engine_destroy(self._h)
            self._h = _vp()
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def request(n, L, waters_angstrom, ions=None, nroots=1, maxsub=20, maxiter=100, ptol=5, corrflag=1,
                precision=PG_FP64, startvec=1, refine=1, key=-1, want_vectors=False):
        """A request with its host arrays (kept alive by the returned tuple)."""
        n = [int(x) for x in np.broadcast_to(n, 3)]
        L = [float(x) for x in np.broadcast_to(L, 3)]
        w = np.ascontiguousarray(waters_angstrom, dtype=np.float64).reshape(-1)
        io = np.ascontiguousarray(ions if ions is not None else np.zeros((0, 4)), dtype=np.float64).reshape(-1)
        vec = np.empty(nroots * n[0] * n[1] * n[2]) if want_vectors else None
        r = Request((C.c_int * 3)(*n), (C.c_double * 3)(*L), len(w) // 9, _d(w) if len(w) else None,
                    len(io) // 4, _d(io) if len(io) else None,
                    SolveParams(nroots, maxsub, maxiter, ptol, corrflag, precision, startvec, refine), key,
                    _d(vec) if want_vectors else None)
        return r, (w, io, vec)

    @staticmethod
    def footprint(req):
        """Device bytes the engine admits the request with."""
        r = req[0] if isinstance(req, tuple) else req
        return lib().pg_request_footprint(C.byref(r))

    def submit(self, req):
        """Submit a request made by Engine.request; returns its id."""
        r, keep = req
        rid = C.c_long(0)
        _check(lib().pg_engine_submit(self._h, C.byref(r), C.byref(rid)))
        self._keep[rid.value] = keep
        return rid.value

    def wait(self, rid, timeout=-1.0):
        """Result of request rid (a dict; 'vectors' holds the eigenvectors when asked for)."""
        out = Result()
        _check(lib().pg_engine_wait(self._h, rid, C.byref(out), timeout))
        d = _result_dict(out)
        keep = self._keep.pop(rid, None)
        if keep is not None and keep[2] is not None:
            d["vectors"] = keep[2].reshape(out.nroots, -1)
        return d

    def poll(self, max_results=64):
        buf = (Result * max_results)()
        k = C.c_int(0)
        _check(lib().pg_engine_poll(self._h, buf, max_results, C.byref(k)))
        res = []
        for i in range(k.value):
            d = _result_dict(buf[i])
            keep = self._keep.pop(buf[i].id, None)
            if keep is not None and keep[2] is not None:
                d["vectors"] = keep[2].reshape(buf[i].nroots, -1)
            res.append(d)
        return res

    def stats(self):
        s = EngineStats()
        _check(lib().pg_engine_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in EngineStats._fields_}
