"""The pure-Python parts of bench.py on the CPU: the arithmetic-type label of
the line, the keys of the measured-traffic table, the workload table, and the
V(r) rate entry driven through stand-ins for the CUDA events and the grid
(no GPU)."""
import importlib.util
import os
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_mixed_dtype_names_the_split(bench):
    assert bench.mixed_dtype("FP16 split (k_hx_f16): xy planes 64x64") == "f64+fp16x3"
    assert bench.mixed_dtype("fused TF32 split (k_hx_fused): ...") == "f64+tf32x3"
    assert bench.mixed_dtype("three axis passes (k_hx_tc)") == "f64+tf32x3"


def test_traffic_table_keys(bench):
    for key, val in bench.KERNEL_TRAFFIC.items():
        assert key[0] in ("gram", "combine", "hx")
        assert isinstance(key[1], tuple) and len(key[1]) == 3
        assert len(key) == (4 if key[0] == "hx" else 5)
        assert isinstance(val, int) and val > 0


def test_workloads_name_their_sizes(bench):
    for name, wl in bench.WORKLOADS.items():
        for k in ("n", "L", "nw", "nroots", "maxsub", "seed"):
            assert k in wl, (name, k)


def test_potential_rate_through_stand_ins(bench):
    class Event:
        clock = 0.0

        def __init__(self, enable_timing=False):
            self.t = None

        def record(self, stream):
            Event.clock += 1.0
            self.t = Event.clock

        def elapsed_time(self, other):
            return other.t - self.t  # ms

    calls = []

    class Grid:
        N = 1000

        def potential(self, tables, stream=None):
            calls.append(stream)

    torch = types.SimpleNamespace(cuda=types.SimpleNamespace(Event=Event, synchronize=lambda: None))
    stream = types.SimpleNamespace(cuda_stream=7)
    r = bench.potential_rate(torch, Grid(), None, 4, stream, reps=5)
    assert calls == [7] * 6  # one warm-up call, then the timed ones, on the launching stream
    assert r["pairs"] == 4000 and r["ms_per_launch"] == pytest.approx(0.2)
    assert r["pairs_per_s"] == pytest.approx(4000 / 0.2e-3)
    assert r["fp64_tflops"] == pytest.approx(r["pairs_per_s"] * bench.POTENTIAL_FLOPS_PER_PAIR / 1e12)
