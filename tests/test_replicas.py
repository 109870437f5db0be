"""Replica plumbing of bench.py on CPU: two gloo ranks agree on the slowest rank's
time and the sum of their work (the path has no exchange step; GPUs run replicas)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench

    elapsed, work = bench.reduce_ranks(dist, 10.0 + rank, 100 * (rank + 1), "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, elapsed, work))


def test_two_rank_reduction():
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 11.0, 300.0), (1, 11.0, 300.0)]
