"""Benchmark of the GB300 eigensolve path (one JSON line on rank 0).

Workload (default, c2): (H2O)24 in a 9 A sphere (seed 2), 64^3 sine-DVR grid
over 40 bohr, lowest 4 states, block 4 (all unconverged roots per H*X
launch), 60-vector subspace.  A step is one complete single point with the
inputs resident on the device: V(r) on the grid from the water-site tables,
diag(H), and the Davidson eigensolve to convergence.

Default form: mixed precision (split-TF32 tensor-core H*X, double-float
subspace products, FP64 subspace eigensolve, Cholesky factors and residual
norms) converged to residual 1e-6, then an FP64 Rayleigh-Ritz step with the
FP64 operator; corrections from the exact-kinetic preconditioner (corrflag 3).
The same run also times the plain FP64 form (residual 1e-8) on the same
problem -- with the same corrections and with the reference's diagonal
correction (corrflag 1) -- and reports |dE| of the mixed eigenvalues against
the FP64 ones.  `value` is mixed solves/s; `e2e` is the same through
pg_cluster_solve with host buffers; `like_for_like` sets the FP64 GPU solve
with the reference's algorithm against the same algorithm on the host cores;
`serving_c4` summarises the serving stream (mixed and FP64 solves/s at
saturation, their ratio, Poisson p50/p99) measured in the same run.
`config` names the workload only (the same in both arms); `solver` gives
each arm's arithmetic, correction and residual.

  python bench.py [--steps K] [--warmup W] [--precision mixed|fp64] [--corrflag 1|3]
  python bench.py --workload c4         # the serving stream through pg_engine_*
  python bench.py --impl reference      # the reference algorithm on the host cores, complete solves
  python bench.py --roofline-only       # the dominant kernels alone (for ncu captures)

Multi-GPU (torchrun, one rank per GPU): replicas only -- every rank solves
its own stream of single points, no data-path collective; value is the
solves of all ranks over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402

WORKLOADS = {
    # name: waters, sphere radius (A), seed, n, L (bohr), nroots, maxsub, ptol
    "c2": dict(nw=24, radius=9.0, seed=2, n=(64, 64, 64), L=(40.0, 40.0, 40.0), nroots=4, maxsub=60, ptol=8),
    "c1": dict(nw=6, radius=6.0, seed=1, n=(32, 32, 32), L=(30.0, 30.0, 30.0), nroots=1, maxsub=20, ptol=8),
    # (H2O)32 + Na+ + Cl- (ion sites seed 33, >= 2.8 A from every O), 96^3 over 48 bohr, 8 states
    "c3": dict(nw=32, radius=10.0, seed=3, ion_seed=33, n=(96, 96, 96), L=(48.0, 48.0, 48.0), nroots=8, maxsub=64,
               ptol=8),
    # (H2O)128 in a 14 A sphere, 160^3 over 64 bohr (4.1M points), 16 states, block 16, maxsub 96
    "c5": dict(nw=128, radius=14.0, seed=5, n=(160, 160, 160), L=(64.0, 64.0, 64.0), nroots=16, maxsub=96,
               ptol=8),
}
A2B = 1.0 / 0.52917720859  # Angstrom -> bohr, the reference's constant


def workload_ions(clusters, wl, waters):
    """Ion list (x, y, z in Angstrom, q) of a workload, or None."""
    if "ion_seed" not in wl:
        return None
    return clusters.place_ions(waters, wl["radius"], wl["ion_seed"])
MIXED_PTOL = 6  # residual threshold of the mixed form before the FP64 Rayleigh-Ritz step
# single-vector H*x products of a full solve by the reference algorithm
# (diagonal correction, FP64), counted by the oracle on the same input
REFERENCE_MATVECS = {"c2": 4500, "c1": 700}  # c3: measured in the same run (the reference-algorithm solve)

# Serving stream: 16 seeded base clusters (H2O)n, n uniform in 8..64, O sites
# in a sphere of radius 9 A (n/24)^(1/3); each request jitters one base by
# 0.1 A / 5 degrees, takes a grid from {48,64,80,96}^3 at spacing 0.615 bohr
# (L = 0.615 (n+1)) and 1-4 states; it warm-starts from its base's vectors.
C4 = dict(nreq=512, nbase=16, grids=(48, 64, 80, 96), spacing=0.615, max_roots=4, maxsub=40, seed=4,
          base_seed=1000, ptol_fp64=8, corrflag=3)


def max_over_ranks(value, ws, device):
    """The largest of the ranks' values (the replica run's slowest rank); the
    only collective of the bench (replicas share no data)."""
    if ws <= 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.out = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def run_ours(args, ws, rank, local):
    import torch
    pg = entry.load_package()
    import importlib
    clusters = importlib.import_module("pisces_gb300.clusters")
    torch.cuda.set_device(local)
    wl = WORKLOADS[args.workload]
    precision = pg.PG_MIXED if args.precision == "mixed" else pg.PG_FP64
    ptol = MIXED_PTOL if precision == pg.PG_MIXED else wl["ptol"]
    waters = clusters.water_cluster(wl["nw"], wl["radius"], wl["seed"])
    ions = workload_ions(clusters, wl, waters)
    tables = pg.WaterTables(waters)
    grid = pg.Grid(wl["n"], wl["L"])
    N = grid.N
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    nroots = wl["nroots"]

    def step(prec=precision, corr=args.corrflag, tol=ptol):
        v = grid.potential(tables, stream=sptr)
        if ions is not None:
            grid.add_ions(v, ions[:, :3] * A2B, ions[:, 3], stream=sptr)
        return grid.solve(v, nroots=nroots, maxsub=wl["maxsub"], maxiter=400, ptol=tol, precision=prec,
                          corrflag=corr, refine=1, stream=sptr)

    def timed(nsteps, **kw):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        lat = []
        a.record(stream)
        for _ in range(nsteps):
            x = torch.cuda.Event(enable_timing=True)
            y = torch.cuda.Event(enable_timing=True)
            x.record(stream)
            out = step(**kw)
            y.record(stream)
            lat.append((x, y))
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b), [x.elapsed_time(y) for x, y in lat], out

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        clocks = ClockSampler(local)
        clocks.start()
        launches0 = pg.lib().pg_kernel_launches()
        total_ms, lat_ms, (ev, vec, st) = timed(args.steps)
        launches = pg.lib().pg_kernel_launches() - launches0
        clk = clocks.stop()
        if ws > 1:
            torch.distributed.barrier()
        # the plain FP64 form on the same problem in the same run: same
        # corrections, residual 10^-ptol of the workload (the drop-in form)
        fp64 = None
        if precision == pg.PG_MIXED:
            step(pg.PG_FP64, args.corrflag, wl["ptol"])
            k = max(1, min(args.steps, 5))
            ms, _, (ev64, _, st64) = timed(k, prec=pg.PG_FP64, tol=wl["ptol"])
            fp64 = {"solves_per_s": 1000.0 * k / ms, "corrflag": args.corrflag, "residual_tol": 10.0 ** -wl["ptol"],
                    "n_matvec": st64["n_matvec"], "eigenvalues": list(map(float, ev64))}
        else:
            ev64, st64 = ev, st
        # the reference's own algorithm (diagonal correction) in FP64 on the GPU, once
        refalg = None
        if not args.no_refalg and not (precision == pg.PG_FP64 and args.corrflag == 1):
            ms, _, (evr, _, str_) = timed(1, prec=pg.PG_FP64, corr=1, tol=wl["ptol"])
            refalg = {"solves_per_s": 1000.0 / ms, "corrflag": 1, "n_matvec": str_["n_matvec"],
                      "n_iter": str_["n_iter"], "eigenvalues": list(map(float, evr))}
        elif precision == pg.PG_FP64 and args.corrflag == 1:
            refalg = {"solves_per_s": 1000.0 * args.steps / total_ms, "corrflag": 1, "n_matvec": st["n_matvec"],
                      "n_iter": st["n_iter"], "eigenvalues": list(map(float, ev))}
    max_ms = max_over_ranks(total_ms, ws, "cuda")
    de = float(np.max(np.abs(np.asarray(ev) - np.asarray(ev64))))

    # end to end through the public host-buffer API: water coordinates in,
    # eigenvalues and eigenvectors out (pg_cluster_solve)
    e2e_ms = None
    d2h = nroots * N * 8 + nroots * 8
    h2d = waters.size * 8 + (ions.size * 8 if ions is not None else 0)
    if not args.no_e2e:
        torch.cuda.synchronize()
        cs = lambda: pg.cluster_solve(wl["n"], wl["L"], waters, ions=ions, nroots=nroots, maxsub=wl["maxsub"],
                                      maxiter=400,
                                      ptol=ptol, precision=precision, corrflag=args.corrflag, refine=1,
                                      want_vectors=True)
        cs()
        t0 = time.perf_counter()
        reps = max(1, min(args.steps, 5))
        for _ in range(reps):
            cs()
        e2e_ms = (time.perf_counter() - t0) * 1000 / reps

    roof = kernel_rooflines(pg, torch, grid, tables, nroots, precision, stream)
    try:
        pot = potential_rate(torch, grid, tables, wl["nw"], stream)
    except Exception as exc:  # reported, not fatal: the line's own numbers are measured above
        pot = {"error": str(exc)}
    hx_plan = grid.hx_plan(nroots)
    return dict(hx_plan=hx_plan, precond_plan=grid.precond_plan(), total_ms=max_ms, lat_ms=lat_ms,
                evals=list(map(float, ev)), evals_fp64=list(map(float, ev64)), de=de, stats=st, fp64=fp64,
                refalg=refalg, clocks=clk, launches=launches, e2e_ms=e2e_ms, h2d=h2d, d2h=d2h, roofline=roof,
                potential=pot, N=N, precision=args.precision, ptol=ptol)


# FP64 operations per (grid point, water) pair of k_potential_dpp besides its
# 4 reciprocal square roots and up to 4 exponentials (charges, induced
# dipoles, Slater cores, damped polarisation, the per-water distances)
POTENTIAL_FLOPS_PER_PAIR = 80


def potential_rate(torch, grid, tables, nwaters, stream, reps=5):
    """V(r) alone (k_potential_dpp) on the bench grid: (grid point, water)
    pairs per second and the FP64 rate they imply, CUDA events on the
    launching stream after one warm-up call."""
    sptr = stream.cuda_stream
    grid.potential(tables, stream=sptr)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(reps):
        grid.potential(tables, stream=sptr)
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    pairs = grid.N * nwaters
    rate = pairs / (ms * 1e-3)
    return {"kernel": "k_potential_dpp", "bound": "fp64", "ms_per_launch": ms, "pairs": pairs,
            "pairs_per_s": rate, "fp64_tflops": rate * POTENTIAL_FLOPS_PER_PAIR / 1e12,
            "flops_per_pair": f"{POTENTIAL_FLOPS_PER_PAIR} FP64 operations besides 4 rsqrt and up to 4 exp",
            "peak_source": "FP64 pipe of this part, about 1.0-1.1 TFLOP/s (a DFMA loop; not in MEASURED_PEAKS.json)"}


GRAM_SHAPE = (40, 4)  # P rows x Q rows of the timed Gram launch: mid-solve basis against a new block


def _time_launches(torch, stream, fn, reps=20, warm=3):
    """Mean device time of fn(i), i = 0 .. reps-1, on stream: after warm
    untimed calls the reps are captured in a CUDA graph and one replay is
    timed with CUDA events, so the host's per-call work (Python, ctypes,
    argument checks) is not part of the time.  Where capture is refused the
    calls are timed back to back."""
    with torch.cuda.stream(stream):
        for i in range(warm):
            fn(i)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    try:
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            for i in range(reps):
                fn(i)
        graph.replay()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            a.record(stream)
            graph.replay()
            b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps
    except RuntimeError:
        torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        a.record(stream)
        for i in range(reps):
            fn(i)
        b.record(stream)
        torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def _rotation(torch, set_bytes):
    """Copies of a launch's operands to cycle through so that consecutive
    launches touch more than twice the L2 between reuses of one copy: each
    launch then streams its operands from HBM, as in the solve."""
    l2 = torch.cuda.get_device_properties(0).L2_cache_size or (129 << 20)
    return max(2, -(-2 * l2 // int(set_bytes)) + 1)


def kernel_rooflines(pg, torch, grid, tables, nb, precision, stream):
    """The dominant kernels of the solve, each timed alone with CUDA events on
    its stream, in the form the solve launches them.  Mixed form: the subspace
    Gram (k_gram_df on double-float twins of both operands, the largest
    single share of a point) and the subspace combine (k_combine_df reading
    twins and writing the twin of its output, the Gram-Schmidt form);
    FP64 form: k_gram and k_combine.  Then the H*X product.  Algorithmic
    bytes: every input vector read once and every output written once
    (Gram, combine); X read, Y written, V read once (H*X)."""
    peaks, which = measured_peaks()
    N = grid.N
    g = torch.Generator(device="cuda").manual_seed(5)
    na, nq = GRAM_SHAPE
    mixed = precision == pg.PG_MIXED
    s = stream.cuda_stream
    k = _rotation(torch, 8.0 * N * (na + 2 * nq))
    sets = []
    for _ in range(k):
        P = torch.randn(na, N, dtype=torch.float64, device="cuda", generator=g)
        Q = torch.randn(nq, N, dtype=torch.float64, device="cuda", generator=g)
        Y = torch.empty(nq, N, dtype=torch.float64, device="cuda")
        if mixed:  # the solve keeps these operands as twins only
            P, Q = pg.split_twin(P, stream=s), pg.split_twin(Q, stream=s)
        sets.append((P, Q, Y, torch.empty_like(Y) if mixed else None))
    out = torch.empty(na * nq, dtype=torch.float64, device="cuda")
    Cm = torch.randn(na, nq, dtype=torch.float64, device="cuda", generator=g)
    if mixed:
        gram_call = lambda i: pg.block_gram_twin(sets[i % k][0], sets[i % k][1], out=out, stream=s)
        comb_call = lambda i: pg.block_combine_twin(sets[i % k][0], Cm, out=sets[i % k][2], out_twin=sets[i % k][3],
                                                    stream=s)
    else:
        gram_call = lambda i: pg.block_gram(sets[i % k][0], sets[i % k][1], precision=precision, out=out, stream=s)
        comb_call = lambda i: pg.block_combine(sets[i % k][0], Cm, precision=precision, out=sets[i % k][2], stream=s)
    rot = f"operands rotated over {k} copies (more than twice the L2 between reuses)"

    def hbm_line(kernel, ms, nbytes, traffic, shape):
        gbs = nbytes / (ms * 1e-3) / 1e9
        return {"kernel": kernel, "bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": gbs / peaks["hbm_gbs"], "peak_source": which, "traffic": traffic, "ms_per_launch": ms,
                "algorithmic_bytes": nbytes, "shape": shape, "l2": rot}

    # Gram: one k_gram_df launch plus its partial-sum reduction per call
    ms = _time_launches(torch, stream, gram_call)
    gram = hbm_line("k_gram_df (twin inputs)" if mixed else "k_gram", ms, 8.0 * N * (na + nq),
                    KERNEL_TRAFFIC.get(("gram", tuple(grid.n), na, nq, precision)),
                    f"{na} x {nq} vectors of {N} points")
    # combine: Y (nq rows) = P^T C, one launch per call; the twin output is
    # written beside Y in the mixed form
    ms = _time_launches(torch, stream, comb_call)
    comb = hbm_line("k_combine_df (twin in, twin out)" if mixed else "k_combine", ms,
                    8.0 * N * (na + (2 if mixed else 1) * nq),
                    KERNEL_TRAFFIC.get(("combine", tuple(grid.n), na, nq, precision)),
                    f"{na} vectors of {N} points combined into {nq}")
    del sets
    v0 = grid.potential(tables, stream=s)
    kh = _rotation(torch, 8.0 * N * (2 * nb + 1))
    hsets = [(v0 if j == 0 else v0.clone(), torch.randn(nb * N, dtype=torch.float64, device="cuda", generator=g),
              torch.empty(nb * N, dtype=torch.float64, device="cuda")) for j in range(kh)]
    # queued back to back (pg_hx_async); the status word is checked once after
    ms = _time_launches(torch, stream, lambda i: grid.hx(hsets[i % kh][0], hsets[i % kh][1], nvec=nb,
                                                         precision=precision, out=hsets[i % kh][2], stream=s,
                                                         wait=False))
    grid.check(stream=s)
    del hsets
    nx, ny, nz = grid.n
    hbytes = 8.0 * N * (2 * nb + 1)
    flops = N * nb * (2 * (nx + ny + nz) + 2)
    hx = {"kernel": f"pg_hx mixed: {grid.hx_plan(nb)}" if mixed else "k_hx_fp64",
          "bound": "hbm" if mixed else "fp64", "ms_per_launch": ms, "algorithmic_bytes": hbytes,
          "vectors_per_launch": nb, "l2": f"operands rotated over {kh} copies (more than twice the L2 between reuses)"}
    if mixed:
        hx.update(achieved=hbytes / (ms * 1e-3) / 1e9, peak=peaks["hbm_gbs"], unit="GB/s",
                  frac=hbytes / (ms * 1e-3) / 1e9 / peaks["hbm_gbs"], peak_source=which,
                  traffic=KERNEL_TRAFFIC.get(("hx", tuple(grid.n), nb, precision)))
    else:
        hx.update(achieved=flops / (ms * 1e-3) / 1e12, peak=1.0, unit="TFLOP/s", frac=flops / (ms * 1e-3) / 1e12,
                  peak_source="FP64 FMA pipe of this GB300, measured with a DFMA loop (not in MEASURED_PEAKS.json)")
    return gram, hx, comb


# dram__bytes_read.sum + dram__bytes_write.sum of one launch of these shapes
# (kernel, grid, vectors in, vectors out, precision) for the subspace kernels
# and (kernel, grid, vectors, precision) for H*X, from an ncu capture of
# `python bench.py --roofline-only [--workload c3]`; shapes not captured
# report null
KERNEL_TRAFFIC = {("gram", (64, 64, 64), 40, 4, 1): 92536832 + 2773248,
                  ("combine", (64, 64, 64), 40, 4, 1): 83933696 + 2898176,
                  ("hx", (64, 64, 64), 4, 1): 10576384 + 0,
                  ("hx", (96, 96, 96), 8, 1): 80203520 + 27850240}


def mixed_dtype(plan):
    """The arithmetic of the mixed form: FP64 everywhere but the H*X
    contractions, which run as three split products on the tensor cores
    (FP16 halves with a per-item scale, or TF32 halves)."""
    return "f64+fp16x3" if plan.startswith("FP16") else "f64+tf32x3"


def cpu_baseline(args, wl, n_matvec_full, budget_s=20.0):
    """The reference algorithm on the host cores (the oracle port, all threads),
    timed on a bounded sample: the first matvecs of the same solve; solves/s is
    extrapolated with the full solve's matvec count."""
    orc = entry.load_oracle()
    import importlib
    entry.load_package()
    clusters = importlib.import_module("pisces_gb300.clusters")
    waters = clusters.water_cluster(wl["nw"], wl["radius"], wl["seed"])
    ions = workload_ions(clusters, wl, waters)
    g = orc.Grid(wl["n"], wl["L"])
    s = orc.dpp_sites(waters)
    t0 = time.perf_counter()
    v = g.potential_dpp(*s[:5])
    if ions is not None:
        g.add_ions(v, (ions[:, :3] * A2B).reshape(-1), ions[:, 3])
    t_pot = time.perf_counter() - t0
    # calibrate: a short sample, then one sized to the budget
    sample = 40
    t0 = time.perf_counter()
    g.solve(v, nstates=wl["nroots"], maxsub=wl["maxsub"], maxiter=400, ptol=wl["ptol"], max_matvec=sample)
    dt = time.perf_counter() - t0
    per = dt / sample
    sample2 = int(max(sample, min(4000, budget_s / max(per, 1e-6))))
    t0 = time.perf_counter()
    _, _, _, nmv = g.solve(v, nstates=wl["nroots"], maxsub=wl["maxsub"], maxiter=400, ptol=wl["ptol"],
                           max_matvec=sample2)
    dt = time.perf_counter() - t0
    per = dt / max(nmv, 1)
    solve_s = t_pot + per * n_matvec_full
    return {"value": 1.0 / solve_s, "unit": "solves/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"V(r) on the full grid + the first {nmv} single-vector matvecs of the reference Davidson "
                      f"(with its subspace work) on {wl['n'][0]}^3, extrapolated to the {n_matvec_full} matvecs "
                      f"of a full solve", "seconds_per_matvec": per, "potential_s": t_pot}


REFERENCE_BUDGET_S = 170.0  # CPU seconds the reference arm may spend on complete solves


def reference_arm(args, wl, cfg):
    """The reference algorithm on the host cores: the oracle port of the
    reference's Davidson (src/Davidson.cpp:61-376, diagonal correction, FP64,
    residual 10^-ptol) and of V(r), with every host thread.  A step is one
    COMPLETE single point (V(r) on the full grid and the solve to
    convergence).  Full solves take about a minute each on the GB300 host, so
    the arm times as many as fit REFERENCE_BUDGET_S (at least one) instead of
    the requested --steps, and says so; its warm-up steps are bounded samples
    (the first 20 H*x of the solve)."""
    orc = entry.load_oracle()
    import importlib
    entry.load_package()
    clusters = importlib.import_module("pisces_gb300.clusters")
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    waters = clusters.water_cluster(wl["nw"], wl["radius"], wl["seed"])
    ions = workload_ions(clusters, wl, waters)
    g = orc.Grid(wl["n"], wl["L"])
    s = orc.dpp_sites(waters)

    def potential():
        v = g.potential_dpp(*s[:5])
        if ions is not None:
            g.add_ions(v, (ions[:, :3] * A2B).reshape(-1), ions[:, 3])
        return v

    def point(max_matvec=0):
        v = potential()
        st, ev, _, nmv = g.solve(v, nstates=wl["nroots"], maxsub=wl["maxsub"], maxiter=2000, ptol=wl["ptol"],
                                 corrflag=1, max_matvec=max_matvec)
        return st, ev, nmv

    for _ in range(args.warmup):
        point(max_matvec=20)
    # the expected length of a complete solve from a bounded sample
    t0 = time.perf_counter()
    _, _, nmv = point(max_matvec=200)
    per = (time.perf_counter() - t0) / max(nmv, 1)
    expect = per * REFERENCE_MATVECS.get(args.workload, 4500)
    nsolves = max(1, min(args.steps, int(REFERENCE_BUDGET_S // max(expect, 1e-9))))
    times, evals, matvecs = [], None, []
    for _ in range(nsolves):
        t0 = time.perf_counter()
        st, ev, nmv = point()
        times.append(time.perf_counter() - t0)
        evals = list(map(float, ev))
        matvecs.append(int(nmv))
    ms = 1000.0 * statistics.mean(times)
    val = 1000.0 / ms
    return {"impl": "reference", "metric": "solves/s", "value": val, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": nsolves, "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": cfg,
            "solver": {"precision": "fp64", "corrflag": 1, "residual_tol": 10.0 ** -wl["ptol"],
                       "algorithm": "the reference's Davidson (diagonal correction) restated in C (oracle port)"},
            "eigenvalues": evals, "n_matvec": matvecs,
            "note": f"{nsolves} complete single point(s) timed (of {args.steps} requested: a complete solve "
                    f"takes ~{expect:.0f} s on these cores); warm-up steps are bounded samples (first 20 H*x)",
            "cpu_baseline": {"value": val, "unit": "solves/s", "cores": threads, "kind": "port",
                             "sample": f"{nsolves} complete reference-algorithm single point(s): V(r) on the "
                                       f"{wl['n'][0]}^3 grid and the Davidson solve to residual "
                                       f"1e-{wl['ptol']} ({matvecs} H*x)"},
            "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def c4_stream(clusters, nreq, seed=C4["seed"]):
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = [int(x) for x in rng.integers(8, 65, size=C4["nbase"])]
    bases = [clusters.water_cluster(n, 9.0 * (n / 24.0) ** (1.0 / 3.0), seed=C4["base_seed"] + i)
             for i, n in enumerate(sizes)]
    reqs = []
    for _ in range(nreq):
        b = int(rng.integers(C4["nbase"]))
        n = int(rng.choice(C4["grids"]))
        nr = int(rng.integers(1, C4["max_roots"] + 1))
        reqs.append(dict(base=b, n=n, L=C4["spacing"] * (n + 1), nroots=nr, waters=clusters.jitter(bases[b], rng)))
    return sizes, reqs


def serve_stream(pg, reqs, precision, rate, slots, batch, window_us):
    """Submits reqs to a fresh engine at Poisson arrivals of the given rate
    (None: all at once) and waits for all; returns results and timings."""
    ptol = MIXED_PTOL if precision == pg.PG_MIXED else C4["ptol_fp64"]
    rng = np.random.Generator(np.random.PCG64(99))
    gaps = rng.exponential(1.0 / rate, size=len(reqs)) if rate else np.zeros(len(reqs))
    arrivals = np.cumsum(gaps) - gaps[0]
    launches0 = pg.lib().pg_kernel_launches()
    with pg.Engine(slots=slots, batch_matvecs=batch, batch_window_us=window_us) as eng:
        made = [pg.Engine.request(q["n"], q["L"], q["waters"], nroots=q["nroots"], maxsub=C4["maxsub"], maxiter=400,
                                  ptol=ptol, corrflag=C4["corrflag"], precision=precision, key=q["base"])
                for q in reqs]
        t0 = time.perf_counter()
        ids = []
        for r, ta in zip(made, arrivals):
            dt = ta - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            ids.append(eng.submit(r))
        res = [eng.wait(i, timeout=600.0) for i in ids]
        wall = time.perf_counter() - t0
        stats = eng.stats()
    lat = sorted(r["latency_seconds"] * 1000.0 for r in res)
    return dict(results=res, wall=wall, solves_per_s=len(reqs) / wall, p50=float(np.percentile(lat, 50)),
                p99=float(np.percentile(lat, 99)), stats=stats, failed=sum(r["status"] != 0 for r in res),
                launches=pg.lib().pg_kernel_launches() - launches0,
                n_matvec=sum(r["stats"]["n_matvec"] for r in res))


def c4_measure(pg, clusters, nreq, warmup, slots, window, unbatched=True):
    """The serving stream through the engine (pg_engine_*): mixed form at
    saturation and at Poisson arrivals (0.7 of saturation), FP64 at
    saturation, on the same requests; returns the measurements."""
    sizes, reqs = c4_stream(clusters, nreq)
    _, warm = c4_stream(clusters, max(3, warmup) * 8, seed=C4["seed"] + 1)
    for prec in (pg.PG_MIXED, pg.PG_FP64):  # warm-up: kernels, grids, allocator
        serve_stream(pg, warm, prec, None, slots, True, window)
    clocks = ClockSampler(0)
    clocks.start()
    mixed = serve_stream(pg, reqs, pg.PG_MIXED, None, slots, True, window)
    clk = clocks.stop()
    fp64 = serve_stream(pg, reqs, pg.PG_FP64, None, slots, True, window)
    unb = serve_stream(pg, reqs, pg.PG_MIXED, None, slots, False, window) if unbatched else None
    rate = 0.7 * mixed["solves_per_s"]
    poisson = serve_stream(pg, reqs, pg.PG_MIXED, rate, slots, True, window)
    de = max(abs(a - b) for rm, rf in zip(mixed["results"], fp64["results"])
             for a, b in zip(rm["evals"], rf["evals"]))
    return dict(sizes=sizes, reqs=reqs, warm=warm, mixed=mixed, fp64=fp64, unbatched=unb, rate=rate,
                poisson=poisson, de=de, clocks=clk)


def c4_summary(m):
    """The stream's figures for the default bench line."""
    return {"requests": len(m["reqs"]), "mixed_solves_per_s": m["mixed"]["solves_per_s"],
            "fp64_solves_per_s": m["fp64"]["solves_per_s"],
            "mixed_over_fp64": m["mixed"]["solves_per_s"] / m["fp64"]["solves_per_s"],
            "poisson": {"rate_per_s": m["rate"], "solves_per_s": m["poisson"]["solves_per_s"],
                        "p50_ms": m["poisson"]["p50"], "p99_ms": m["poisson"]["p99"]},
            "saturation_latency_ms": {"p50": m["mixed"]["p50"], "p99": m["mixed"]["p99"]},
            "max_abs_dE_vs_fp64": m["de"], "failed": m["mixed"]["failed"] + m["fp64"]["failed"],
            "warm_starts": m["mixed"]["stats"]["warm_starts"], "clocks": m["clocks"],
            "workload": f"{len(m['reqs'])} single points, grids {list(C4['grids'])}^3, 1-{C4['max_roots']} states, "
                        f"seed {C4['seed']}; mixed residual 1e-{MIXED_PTOL} + FP64 Rayleigh-Ritz, "
                        f"FP64 residual 1e-{C4['ptol_fp64']}, corrflag {C4['corrflag']} both"}


def run_c4(args):
    """The serving stream as its own bench line (`--workload c4`)."""
    import torch
    pg = entry.load_package()
    import importlib
    clusters = importlib.import_module("pisces_gb300.clusters")
    torch.cuda.set_device(0)
    nreq = args.requests
    slots, window = args.slots, args.window_us
    m = c4_measure(pg, clusters, nreq, args.warmup, slots, window)
    mixed, fp64, poisson, reqs, sizes = m["mixed"], m["fp64"], m["poisson"], m["reqs"], m["sizes"]
    h2d = sum(q["waters"].size * 8 for q in reqs) / nreq
    d2h = sum(q["nroots"] * 8 for q in reqs) / nreq
    cfg = {"workload": f"c4: {nreq} single points from {C4['nbase']} base (H2O)n clusters (n = {sorted(sizes)}), "
                       f"grids {list(C4['grids'])}^3 at {C4['spacing']} bohr, 1-{C4['max_roots']} states, "
                       f"maxsub {C4['maxsub']}, warm start per base cluster",
           "seed": C4["seed"], "slots": slots, "batch_window_us": window,
           "l2": "per-solve working sets of 48^3-96^3 grids; no flush (requests differ)"}
    line = {"metric": "solves/s", "value": mixed["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": nreq,
            "warmup": len(m["warm"]), "ms_per_step": 1000.0 * mixed["wall"] / nreq, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+fp16x3|tf32x3", "data": "synthetic", "config": cfg,
            "solver": {"precision": "mixed", "corrflag": C4["corrflag"], "residual_tol": 10.0 ** -MIXED_PTOL,
                       "fp64_residual_tol": 10.0 ** -C4["ptol_fp64"]},
            "latency_ms": {"p50": mixed["p50"], "p99": mixed["p99"], "at": "saturation (all submitted at once)"},
            "poisson": {"rate_per_s": m["rate"], "solves_per_s": poisson["solves_per_s"], "p50_ms": poisson["p50"],
                        "p99_ms": poisson["p99"]},
            "fp64_gpu": {"solves_per_s": fp64["solves_per_s"], "p50_ms": fp64["p50"], "p99_ms": fp64["p99"],
                         "n_matvec": fp64["n_matvec"]},
            "mixed_over_fp64": mixed["solves_per_s"] / fp64["solves_per_s"],
            "unbatched_mixed_solves_per_s": m["unbatched"]["solves_per_s"],
            "max_abs_dE_vs_fp64": m["de"], "failed": mixed["failed"] + fp64["failed"],
            "engine": mixed["stats"], "n_matvec": mixed["n_matvec"], "clocks": m["clocks"],
            "gpu_launches": mixed["launches"],
            "e2e": {"value": mixed["solves_per_s"], "unit": "solves/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "note": "the engine takes host coordinates and returns host "
                                                      "eigenvalues: value is already end to end"}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS) + ["c4"])
    ap.add_argument("--requests", type=int, default=C4["nreq"], help="c4: requests in the timed stream")
    ap.add_argument("--slots", type=int, default=16, help="c4: engine slots")
    ap.add_argument("--window-us", type=int, default=200, help="c4: matvec batching window")
    ap.add_argument("--corrflag", type=int, default=3, choices=[1, 3],
                    help="1: the reference's diagonal (Davidson) correction; 3: exact-kinetic preconditioner")
    ap.add_argument("--no-refalg", action="store_true",
                    help="skip the FP64 solve with the reference's diagonal correction")
    ap.add_argument("--roofline-only", action="store_true", help="time the dominant kernels only")
    ap.add_argument("--maxsub", type=int, default=0, help="override the workload's subspace size")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c4", action="store_true", help="skip the serving-stream summary of the default line")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.workload == "c4":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the serving stream has no reference counterpart "
                                                                  "(the reference solves one point at a time)"}))
            return
        if rank == 0:
            run_c4(args)
        return
    wl = dict(WORKLOADS[args.workload])
    if args.maxsub:
        wl["maxsub"] = args.maxsub
    WORKLOADS[args.workload] = wl
    cfg = {"workload": f"{args.workload}: (H2O){wl['nw']}{' + Na+ + Cl-' if 'ion_seed' in wl else ''} "
                       f"{wl['n'][0]}^3 sine-DVR over {wl['L'][0]} bohr, "
                       f"{wl['nroots']} states, block {wl['nroots']}, maxsub {wl['maxsub']}",
           "grid": list(wl["n"]), "box_bohr": list(wl["L"]), "waters": wl["nw"], "seed": wl["seed"],
           "nroots": wl["nroots"], "maxsub": wl["maxsub"], "l2": "working set (B, Z: 2 x maxsub x N doubles) "
                                                                 "larger than L2; no flush"}

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(reference_arm(args, wl, cfg)))
        return

    import torch
    if args.roofline_only:
        pg = entry.load_package()
        import importlib
        clusters = importlib.import_module("pisces_gb300.clusters")
        torch.cuda.set_device(local)
        grid = pg.Grid(wl["n"], wl["L"])
        tables = pg.WaterTables(clusters.water_cluster(wl["nw"], wl["radius"], wl["seed"]))
        prec = pg.PG_MIXED if args.precision == "mixed" else pg.PG_FP64
        gram, hx, comb = kernel_rooflines(pg, torch, grid, tables, wl["nroots"], prec, torch.cuda.Stream())
        print(json.dumps({"roofline": gram, "roofline_combine": comb, "roofline_hx": hx, "config": cfg}))
        return
    if ws > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    r = run_ours(args, ws, rank, local)
    solves = ws * args.steps
    value = solves / (r["total_ms"] / 1000.0)
    lat = sorted(r["lat_ms"])
    p50 = float(np.percentile(lat, 50))
    p99 = float(np.percentile(lat, 99))
    line = {"metric": "solves/s", "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["total_ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else mixed_dtype(r["hx_plan"]), "data": "synthetic", "config": cfg,
            "solver": {"precision": args.precision, "corrflag": args.corrflag, "residual_tol": 10.0 ** -r["ptol"],
                       "refine": "FP64 Rayleigh-Ritz step" if args.precision == "mixed" else None,
                       "hx_kernel": r["hx_plan"],
                       "preconditioner": r["precond_plan"] if args.corrflag == 3 else None},
            "latency_ms": {"p50": p50, "p99": p99},
            "eigenvalues": r["evals"], "max_abs_dE_vs_fp64": r["de"],
            "solve": {k: r["stats"][k] for k in ("n_matvec", "n_iter", "n_restart", "nconv", "seconds",
                                                 "host_eig_seconds", "device_wait_seconds")},
            "roofline": r["roofline"][0], "roofline_combine": r["roofline"][2],
            "roofline_hx": r["roofline"][1], "potential": r["potential"], "clocks": r["clocks"],
            "gpu_launches": r["launches"]}
    if r["fp64"]:
        line["fp64_gpu"] = dict(r["fp64"], solves_per_s=ws * r["fp64"]["solves_per_s"])
        line["mixed_over_fp64"] = value / line["fp64_gpu"]["solves_per_s"]
    if r["refalg"]:
        line["fp64_gpu_reference_algorithm"] = dict(r["refalg"], solves_per_s=ws * r["refalg"]["solves_per_s"])
    if r["e2e_ms"] is not None:
        line["e2e"] = {"value": ws * 1000.0 / r["e2e_ms"], "unit": "solves/s", "h2d_bytes_per_step": r["h2d"],
                       "d2h_bytes_per_step": r["d2h"],
                       "path": "pg_cluster_solve: host water coordinates in, host eigenvalues and eigenvectors out"}
    if rank == 0 and not args.no_cpu_baseline:
        nfull = r["refalg"]["n_matvec"] if r["refalg"] else REFERENCE_MATVECS.get(args.workload)
        line["cpu_baseline"] = cpu_baseline(args, WORKLOADS[args.workload], nfull)
        if r["refalg"]:
            # the same algorithm on both sides: the reference's diagonal
            # correction in FP64 to the same residual, GPU against host cores
            a, b = line["fp64_gpu_reference_algorithm"]["solves_per_s"], line["cpu_baseline"]["value"]
            line["like_for_like"] = {"fp64_gpu_reference_algorithm_solves_per_s": a,
                                     "cpu_reference_algorithm_solves_per_s": b, "ratio": a / b,
                                     "note": "reference algorithm (corrflag 1, FP64, residual "
                                             f"1e-{WORKLOADS[args.workload]['ptol']}) on both; the headline value "
                                             "also changes the algorithm (corrflag 3, mixed form)"}
    if rank == 0 and ws == 1 and args.workload == "c2" and not args.no_c4:
        import importlib
        pg = entry.load_package()
        clusters = importlib.import_module("pisces_gb300.clusters")
        line["serving_c4"] = c4_summary(c4_measure(pg, clusters, args.requests, args.warmup, args.slots,
                                                   args.window_us, unbatched=False))
    if ws > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
