"""Replica bookkeeping across two processes (gloo on CPU, world size 2).

The path needs no data-path collective; the only cross-rank steps are the
barrier and the max over ranks of the timed interval, which are checked here
on the CPU the same way bench.py uses them over NCCL on GPUs.
"""

from __future__ import annotations

import importlib
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, pkg_name: str, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rep = importlib.import_module(pkg_name + ".replicas")
        ms = rep.slowest_ms(10.0 + 5.0 * rank, world)          # rank 1 is slower
        dist.barrier()
        value = rep.job_gsps(1_000_000_000, world, ms)
        out.put((rank, ms, value, rep.replica_seed_offset(rank)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_value(pkg):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, pkg.__name__, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank sees the slowest rank's time; value counts both ranks' units
    assert [r[1] for r in res] == [15.0, 15.0]
    assert res[0][2] == pytest.approx(2 * 1e9 / 15e-3 / 1e9)
    assert res[0][2] == res[1][2]
    # replicas draw different inputs
    assert res[0][3] != res[1][3]


def test_single_rank_needs_no_process_group(pkg):
    rep = importlib.import_module(pkg.__name__ + ".replicas")
    assert rep.slowest_ms(7.5, 1) == 7.5
    assert rep.job_gsps(201_326_592, 1, 1.0) == pytest.approx(201.326592)
