"""Multi-rank bookkeeping of bench.py (replicas: one solve per GPU) on CPU
with the gloo backend, world size 2."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from fdtd_gb300 import replicas  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, lr, w = replicas.dist_env()
        assert (r, lr, w) == (rank, rank, world)
        replicas.barrier(dist)
        units, secs = replicas.aggregate(1000.0 * (rank + 1), 0.5 + rank, dist, device="cpu")
        out.put((rank, units, secs))
    finally:
        dist.destroy_process_group()


def test_aggregate_sums_units_and_takes_slowest_rank():
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
    assert res == [(0, 3000.0, 1.5), (1, 3000.0, 1.5)]


def test_single_process_aggregate_is_identity():
    assert replicas.aggregate(5.0, 2.0, None) == (5.0, 2.0)
