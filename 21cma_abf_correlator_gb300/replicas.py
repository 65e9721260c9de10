"""Replica bookkeeping for runs with one process per GPU.

The FX path shards over time: every integration is independent, so N processes
each run their own integrations and exchange nothing on the data path. The only
cross-process steps are the bench's barrier and the max over ranks of the timed
interval; `value` is the units all ranks processed divided by that time. These
helpers work with any torch.distributed backend (NCCL on GPUs, gloo on CPUs).
"""

from __future__ import annotations


def replica_seed_offset(rank: int) -> int:
    """Each replica generates its own inputs: seed offset = rank."""
    return rank


def slowest_ms(ms_local: float, world: int, device: str = "cpu") -> float:
    """Max over ranks of a per-rank time (every rank gets the result)."""
    if world <= 1:
        return float(ms_local)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_gsps(units_per_rank_step: int, world: int, ms_per_step: float) -> float:
    """Whole-job throughput: all ranks' units per step over the slowest rank's time."""
    return units_per_rank_step * world / (ms_per_step * 1e-3) / 1e9
