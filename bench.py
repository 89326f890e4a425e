"""Benchmark of the GB300 eigensolve path (one JSON line on rank 0).

Workload (default): (H2O)24 in a 9 A sphere (seed 2), 64^3 sine-DVR grid over
40 bohr, lowest 4 states, block 4 (all unconverged roots per H*X launch),
60-vector subspace.  A step is one complete single point: V(r) on the grid
from the water-site tables, diag(H), and the Davidson eigensolve to
convergence.  The FP64 form converges to residual 1e-8 (|dE| far below
1e-8 Eh); the mixed form converges to a looser residual with split-TF32
tensor-core H*X and finishes with an FP64 Rayleigh-Ritz step.

  python bench.py [--steps K] [--warmup W] [--precision mixed|fp64]
  python bench.py --impl reference      # the reference algorithm on the host cores

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
}
MIXED_PTOL = 6  # residual threshold of the mixed form before the FP64 Rayleigh-Ritz step

# Serving stream: 16 seeded base clusters (H2O)n, n uniform in 8..64, O sites
# in a sphere of radius 9 A (n/24)^(1/3); each request jitters one base by
# 0.1 A / 5 degrees, takes a grid from {48,64,80,96}^3 at spacing 0.615 bohr
# (L = 0.615 (n+1)) and 1-4 states; it warm-starts from its base's vectors.
C4 = dict(nreq=512, nbase=16, grids=(48, 64, 80, 96), spacing=0.615, max_roots=4, maxsub=40, seed=4,
          base_seed=1000, ptol_fp64=8, corrflag=3)


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
    tables = pg.WaterTables(waters)
    grid = pg.Grid(wl["n"], wl["L"])
    N = grid.N
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    nroots = wl["nroots"]

    def step():
        v = grid.potential(tables, stream=sptr)
        return grid.solve(v, nroots=nroots, maxsub=wl["maxsub"], maxiter=400, ptol=ptol, precision=precision,
                          corrflag=args.corrflag, refine=1, stream=sptr)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            ev, vec, st = step()
        ev_ref, _, st_ref = ev, vec, st
        if precision == pg.PG_MIXED:  # FP64 answer of the same problem, for the error statement
            v = grid.potential(tables, stream=sptr)
            ev_ref, _, st_ref = grid.solve(v, nroots=nroots, maxsub=wl["maxsub"], maxiter=400, ptol=wl["ptol"],
                                           precision=pg.PG_FP64, corrflag=args.corrflag, stream=sptr)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        clocks = ClockSampler(local)
        clocks.start()
        launches0 = pg.lib().pg_kernel_launches()
        lat = []
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ev, vec, st = step()
            b.record(stream)
            lat.append((a, b))
        e1.record(stream)
        torch.cuda.synchronize()
        launches = pg.lib().pg_kernel_launches() - launches0
        clk = clocks.stop()
    total_ms = e0.elapsed_time(e1)
    lat_ms = [a.elapsed_time(b) for a, b in lat]
    max_ms = total_ms
    if ws > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        max_ms = float(t.item())
    de = float(np.max(np.abs(np.asarray(ev) - np.asarray(ev_ref))))

    # end to end through the public host-buffer API: water coordinates in,
    # eigenvalues and eigenvectors out (pg_cluster_solve)
    e2e_ms = None
    d2h = nroots * N * 8
    h2d = waters.size * 8
    if not args.no_e2e:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = max(1, min(args.steps, 3))
        for _ in range(reps):
            pg.cluster_solve(wl["n"], wl["L"], waters, nroots=nroots, maxsub=wl["maxsub"], maxiter=400, ptol=ptol,
                             precision=precision, corrflag=args.corrflag, refine=1, want_vectors=True)
        e2e_ms = (time.perf_counter() - t0) * 1000 / reps

    # dominant kernel: H*X on a block of nroots vectors, timed with CUDA events on its stream
    roof = hx_roofline(pg, torch, grid, tables, nroots, precision, stream)
    return dict(total_ms=max_ms, lat_ms=lat_ms, evals=list(map(float, ev)), evals_fp64=list(map(float, ev_ref)),
                de=de, stats=st, stats_fp64=st_ref, clocks=clk, launches=launches, e2e_ms=e2e_ms, h2d=h2d, d2h=d2h,
                roofline=roof, N=N, precision=args.precision, ptol=ptol)


def hx_roofline(pg, torch, grid, tables, nb, precision, stream):
    v = grid.potential(tables, stream=stream.cuda_stream)
    X = torch.randn(nb * grid.N, dtype=torch.float64, device="cuda")
    Y = torch.empty_like(X)
    nx, ny, nz = grid.n
    reps = 20
    with torch.cuda.stream(stream):
        for _ in range(3):
            grid.hx(v, X, nvec=nb, precision=precision, out=Y, stream=stream.cuda_stream)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            grid.hx(v, X, nvec=nb, precision=precision, out=Y, stream=stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    N = grid.N
    flops = N * nb * (2 * (nx + ny + nz) + 2)
    bytes_ = 8 * N * (2 * nb + 1)
    peaks, which = measured_peaks()
    if precision == pg.PG_MIXED:
        achieved = bytes_ / (ms * 1e-3) / 1e9
        peak = peaks["hbm_gbs"]
        return {"kernel": "pg_hx mixed (split-TF32 tcgen05)", "bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": which, "traffic": None,
                "ms_per_launch": ms, "algorithmic_bytes": bytes_, "vectors_per_launch": nb}
    achieved = flops / (ms * 1e-3) / 1e12
    peak = 1.0  # FP64 FMA pipe of this GB300, measured (DFMA loop, 1.00-1.01 TFLOP/s)
    return {"kernel": "k_hx_fp64", "bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "peak_source": "measured FP64 DFMA throughput (not in MEASURED_PEAKS.json)",
            "traffic": None, "ms_per_launch": ms, "algorithmic_flops": flops, "vectors_per_launch": nb}


def cpu_baseline(args, wl, n_matvec_full, budget_s=20.0):
    """The reference algorithm on the host cores (the oracle port, all threads),
    timed on a bounded sample: the first matvecs of the same solve; solves/s is
    extrapolated with the full solve's matvec count."""
    orc = entry.load_oracle()
    import importlib
    entry.load_package()
    clusters = importlib.import_module("pisces_gb300.clusters")
    waters = clusters.water_cluster(wl["nw"], wl["radius"], wl["seed"])
    g = orc.Grid(wl["n"], wl["L"])
    s = orc.dpp_sites(waters)
    t0 = time.perf_counter()
    v = g.potential_dpp(*s[:5])
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


def run_c4(args):
    """The serving stream through the engine (pg_engine_*): mixed form at
    saturation and at Poisson arrivals, FP64 at saturation, same requests."""
    import torch
    pg = entry.load_package()
    import importlib
    clusters = importlib.import_module("pisces_gb300.clusters")
    torch.cuda.set_device(0)
    nreq = args.requests
    sizes, reqs = c4_stream(clusters, nreq)
    _, warm = c4_stream(clusters, max(3, args.warmup) * 8, seed=C4["seed"] + 1)
    slots, window = args.slots, args.window_us
    for prec in (pg.PG_MIXED, pg.PG_FP64):  # warm-up: kernels, grids, allocator
        serve_stream(pg, warm, prec, None, slots, True, window)
    clocks = ClockSampler(0)
    clocks.start()
    mixed = serve_stream(pg, reqs, pg.PG_MIXED, None, slots, True, window)
    clk = clocks.stop()
    fp64 = serve_stream(pg, reqs, pg.PG_FP64, None, slots, True, window)
    unbatched = serve_stream(pg, reqs, pg.PG_MIXED, None, slots, False, window)
    rate = 0.7 * mixed["solves_per_s"]
    poisson = serve_stream(pg, reqs, pg.PG_MIXED, rate, slots, True, window)
    de = max(abs(a - b) for rm, rf in zip(mixed["results"], fp64["results"])
             for a, b in zip(rm["evals"], rf["evals"]))
    h2d = sum(q["waters"].size * 8 for q in reqs) / nreq
    d2h = sum(q["nroots"] * 8 for q in reqs) / nreq
    cfg = {"workload": f"c4: {nreq} single points from {C4['nbase']} base (H2O)n clusters (n = {sorted(sizes)}), "
                       f"grids {list(C4['grids'])}^3 at {C4['spacing']} bohr, 1-{C4['max_roots']} states, "
                       f"maxsub {C4['maxsub']}, warm start per base cluster",
           "seed": C4["seed"], "slots": slots, "batch_window_us": window, "corrflag": C4["corrflag"],
           "precision": "mixed", "residual_tol": 10.0 ** -MIXED_PTOL, "fp64_residual_tol": 10.0 ** -C4["ptol_fp64"],
           "l2": "per-solve working sets of 48^3-96^3 grids; no flush (requests differ)"}
    line = {"metric": "solves/s", "value": mixed["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": nreq,
            "warmup": len(warm), "ms_per_step": 1000.0 * mixed["wall"] / nreq, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+tf32x3", "data": "synthetic", "config": cfg,
            "latency_ms": {"p50": mixed["p50"], "p99": mixed["p99"], "at": "saturation (all submitted at once)"},
            "poisson": {"rate_per_s": rate, "solves_per_s": poisson["solves_per_s"], "p50_ms": poisson["p50"],
                        "p99_ms": poisson["p99"]},
            "fp64_gpu": {"solves_per_s": fp64["solves_per_s"], "p50_ms": fp64["p50"], "p99_ms": fp64["p99"],
                         "n_matvec": fp64["n_matvec"]},
            "mixed_over_fp64": mixed["solves_per_s"] / fp64["solves_per_s"],
            "unbatched_mixed_solves_per_s": unbatched["solves_per_s"],
            "max_abs_dE_vs_fp64": de, "failed": mixed["failed"] + fp64["failed"],
            "engine": mixed["stats"], "n_matvec": mixed["n_matvec"], "clocks": clk, "gpu_launches": mixed["launches"],
            "e2e": {"value": mixed["solves_per_s"], "unit": "solves/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "note": "the engine takes host coordinates and returns host "
                                                      "eigenvalues: value is already end to end"}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS) + ["c4"])
    ap.add_argument("--requests", type=int, default=C4["nreq"], help="c4: requests in the timed stream")
    ap.add_argument("--slots", type=int, default=16, help="c4: engine slots")
    ap.add_argument("--window-us", type=int, default=200, help="c4: matvec batching window")
    ap.add_argument("--corrflag", type=int, default=1, choices=[1, 3],
                    help="1: the reference's diagonal (Davidson) correction; 3: exact-kinetic preconditioner")
    ap.add_argument("--maxsub", type=int, default=0, help="override the workload's subspace size")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
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
    cfg = {"workload": f"{args.workload}: (H2O){wl['nw']} {wl['n'][0]}^3 sine-DVR over {wl['L'][0]} bohr, "
                       f"{wl['nroots']} states, block {wl['nroots']}, maxsub {wl['maxsub']}",
           "grid": list(wl["n"]), "box_bohr": list(wl["L"]), "waters": wl["nw"], "seed": wl["seed"],
           "nroots": wl["nroots"], "maxsub": wl["maxsub"], "l2": "working set (B, Z: 2 x maxsub x N doubles) "
                                                                 "larger than L2; no flush"}

    if args.impl == "reference":
        if rank != 0:
            return
        # matvec count of a full solve of this workload (reference algorithm,
        # FP64); measured by the GPU FP64 path, which follows the same algorithm
        n_full = 3656 if args.workload == "c2" else 700
        steps = []
        for _ in range(args.warmup + args.steps):
            steps.append(cpu_baseline(args, wl, n_full, budget_s=8.0))
        timed = steps[args.warmup:]
        val = statistics.median(s["value"] for s in timed)
        line = {"impl": "reference", "metric": "solves/s", "value": val, "unit": "solves/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / val, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": cfg, "cpu_baseline": dict(timed[-1], value=val),
                "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
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
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64+tf32x3",
            "data": "synthetic", "config": dict(cfg, precision=args.precision, residual_tol=10.0 ** -r["ptol"],
                                                  corrflag=args.corrflag),
            "latency_ms": {"p50": p50, "p99": p99},
            "eigenvalues": r["evals"], "max_abs_dE_vs_fp64": r["de"],
            "solve": {k: r["stats"][k] for k in ("n_matvec", "n_iter", "n_restart", "nconv", "seconds",
                                                 "host_eig_seconds", "device_wait_seconds")},
            "roofline": r["roofline"], "clocks": r["clocks"], "gpu_launches": r["launches"]}
    if r["e2e_ms"] is not None:
        line["e2e"] = {"value": ws * 1000.0 / r["e2e_ms"], "unit": "solves/s", "h2d_bytes_per_step": r["h2d"],
                       "d2h_bytes_per_step": r["d2h"]}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, WORKLOADS[args.workload], r["stats_fp64"]["n_matvec"])
    if ws > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
