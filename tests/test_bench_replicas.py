"""The replica aggregation of bench.py on world_size 2 (gloo, CPU): the step
time is the maximum over ranks and the value counts every rank's units."""
from __future__ import annotations

import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.combine_ranks(10.0 * (rank + 1), 64, "cpu")
    q.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_combine_ranks_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, ms, value in out:
        assert ms == pytest.approx(20.0)              # max over ranks
        assert value == pytest.approx(2 * 64 / 0.020)  # both ranks' units over that time


def test_combine_ranks_single(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    ms, value = bench.combine_ranks(4.0, 8, "cpu")
    assert ms == 4.0 and value == pytest.approx(2000.0)
