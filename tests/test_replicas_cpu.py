"""Multi-GPU bench path on CPU: two gloo ranks run the replica logic the
bench uses under torchrun (rank environment, barrier, max over ranks of the
timed region), without a GPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    w, r, local = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    dist.barrier()
    got = bench.max_over_ranks(10.0 * (r + 1), w, "cpu")
    dist.barrier()
    out.put((r, w, local, got))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _, _ in res] == [0, 1]
    assert all(w == 2 for _, w, _, _ in res)
    assert all(got == 20.0 for _, _, _, got in res)  # the slower rank's time, on both ranks


def test_single_rank_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
