"""Autotuner of the mixed-form H*X launch parameters (run on a GB300).

    python pisces-1_gb300/tune_hx.py [--sizes 32 48 64 80 96 160] [--nvec 1 2 4 8 16] [--out FILE]

For every cubic grid size n and block size nvec it times each candidate --
the fused kernels (TF32 and FP16 split) with z lag 1, 2, 3 and one CTA per
SM or half as many; the three axis passes in serial and pipelined form -- with CUDA events over
back-to-back launches after warm-up, cycling through copies of X, V and Y
that exceed twice the L2 between reuses (every launch streams its operands
from HBM, as the bench's roofline does), checks each against the FP64
product within the mixed form's bound, and writes the fastest to hx_tuned.tsv beside this file.  The
build compiles that table into the library; each mixed H*X call looks up
its grid size and the nearest tuned block size.
"""
from __future__ import annotations

import argparse
import importlib.util
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def load_package():
    if "pisces_gb300" in sys.modules:
        return sys.modules["pisces_gb300"]
    spec = importlib.util.spec_from_file_location("pisces_gb300", os.path.join(HERE, "__init__.py"),
                                                  submodule_search_locations=[HERE])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["pisces_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def time_us(torch, fn, reps=20, warm=4):
    """Mean device time of fn() in microseconds: after warm calls the reps
    are captured in a CUDA graph on a side stream and one replay is timed
    with CUDA events (no host overhead per call); where capture is refused,
    back-to-back calls on the current stream."""
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        for _ in range(warm):
            fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    try:
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=st):
            for _ in range(reps):
                fn()
        graph.replay()
        torch.cuda.synchronize()
        with torch.cuda.stream(st):
            a.record(st)
            graph.replay()
            b.record(st)
        torch.cuda.synchronize()
        return 1000.0 * a.elapsed_time(b) / reps
    except RuntimeError:
        torch.cuda.synchronize()
    cur = torch.cuda.current_stream()
    a.record(cur)
    for _ in range(reps):
        fn()
    b.record(cur)
    torch.cuda.synchronize()
    return 1000.0 * a.elapsed_time(b) / reps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", type=int, nargs="+", default=[32, 48, 64, 80, 96, 160])
    ap.add_argument("--nvec", type=int, nargs="+", default=[1, 2, 4, 8, 16])
    ap.add_argument("--out", default=os.path.join(HERE, "hx_tuned.tsv"))
    args = ap.parse_args()
    import torch
    pg = load_package()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    candidates = ([(3, lag, c, 0) for lag in (1, 2, 3) for c in (0, sms // 2)] +
                  [(2, lag, c, 0) for lag in (1, 2, 3) for c in (0, sms // 2)] + [(1, 0, 0, 1), (1, 0, 0, 2)])
    lines = ["# n nvec kind lag ctas form  us_tuned us_default  (kind 1: three axis passes, 2: fused, "
             "3: fused with the FP16 split; "
             "form 1 serial, 2 pipelined; 0 = default)",
             f"# measured on {torch.cuda.get_device_name(0)}, {sms} SMs, by pisces-1_gb300/tune_hx.py"]
    g0 = torch.Generator(device="cuda").manual_seed(12)
    for n in args.sizes:
        grid = pg.Grid((n, n, n), (0.615 * (n + 1),) * 3)
        N = grid.N
        v = torch.randn(N, dtype=torch.float64, device="cuda", generator=g0)
        l2 = torch.cuda.get_device_properties(0).L2_cache_size or (129 << 20)
        for nv in args.nvec:
            # copies of the operands to cycle through, more than twice the L2
            # between reuses of one copy, so that every launch streams them
            # from HBM (the roofline's condition)
            k = max(2, -(-2 * l2 // int(8 * N * (2 * nv + 1))) + 1)
            sets = [(torch.randn(nv * N, dtype=torch.float64, device="cuda", generator=g0),
                     torch.empty(nv * N, dtype=torch.float64, device="cuda"),
                     v if c == 0 else v.clone()) for c in range(k)]
            X, Y, _ = sets[0]
            ref = grid.hx(v, X, nvec=nv, precision=pg.PG_FP64)
            scale = float(ref.abs().max())
            turn = [0]

            def call():
                Xc, Yc, vc = sets[turn[0] % k]
                turn[0] += 1
                grid.hx(vc, Xc, nvec=nv, precision=pg.PG_MIXED, out=Yc, wait=False)

            grid.set_hx_params(0, 0, 0, 0)
            t_default = time_us(torch, call)
            grid.check()
            best = None
            for kind, lag, ctas, form in candidates:
                try:
                    grid.set_hx_params(kind, lag, ctas, form)
                except pg.PiscesError:
                    continue  # the fused kernel does not take this grid
                if form == 2 and n > 112:
                    continue  # the pipelined form needs one K chunk
                t = time_us(torch, call)
                grid.check()
                grid.hx(v, X, nvec=nv, precision=pg.PG_MIXED, out=Y)
                err = float((Y - ref).abs().max()) / scale
                if err > 2e-5:
                    raise RuntimeError(f"n={n} nvec={nv} {(kind, lag, ctas, form)}: error {err:.2e}")
                if best is None or t < best[0]:
                    best = (t, kind, lag, ctas, form)
            grid.set_hx_params(0, 0, 0, 0)
            t, kind, lag, ctas, form = best
            lines.append(f"{n} {nv} {kind} {lag} {ctas} {form}  {t:.1f} {t_default:.1f}")
            print(lines[-1], flush=True)
            del X, Y, ref, sets
        grid.close()
    with open(args.out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", args.out)


if __name__ == "__main__":
    main()
