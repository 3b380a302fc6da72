"""Replica bookkeeping of multi-GPU runs, on CPU: two gloo ranks with different work and times;
the whole-job rate is the summed work over the slowest rank's time, on every rank."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "hermite-teno_gb300"))
    import torch
    import torch.distributed as dist

    from hteno import replicas

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = 1000.0 * (rank + 1)
        secs = 2.0 + rank
        rate = replicas.aggregate_rate(torch, units, secs)
        mx = replicas.reduce(torch, float(rank), "max")
        out.put((rank, rate, mx, replicas.world_info()[:2]))
    finally:
        dist.destroy_process_group()


def test_replica_rate_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, mx, (w, r) in res:
        assert rate == pytest.approx(3000.0 / 3.0) and mx == 1.0 and w == 2 and r == rank


def test_replica_rate_single_process():
    import sys

    import torch

    from hteno import replicas

    assert replicas.aggregate_rate(torch, 10.0, 2.0) == 5.0
