"""The bench's N > 1 path on CPU: two gloo ranks, as torchrun would start
them, agree on the slowest rank's time through bench.Replicas (replicas
only: no data-path collective)."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    rep = bench.Replicas()
    rep.barrier()
    out.put((rank, rep.world, rep.max(10.0 + 5.0 * rank)))
    rep.barrier()
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 15.0), (1, 2, 15.0)]


def test_single_process_needs_no_process_group(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    sys.path.insert(0, str(ROOT))
    import bench
    rep = bench.Replicas()
    assert rep.world == 1 and rep.max(3.5) == 3.5
    rep.barrier()
