"""Replica aggregation of bench.py under torch.distributed (world_size 2,
gloo on CPU): every rank sees the slowest rank's time and the total work."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.barrier_max(100.0 + 10.0 * rank, world)
    work = bench.barrier_sum(3.0 + rank, world)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, ms, work))


def test_two_replicas_gloo():
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 110.0, 7.0), (1, 110.0, 7.0)]
