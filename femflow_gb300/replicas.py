"""Replica bookkeeping for runs on several GPUs of one node (one process per GPU).

The MLS-MPM substep has no exchange step between scenes, so N GPUs run N independent replicas
(or disjoint shares of a batch of independent scenes) and nothing crosses GPUs on the data path.
Only the measurement is collective: a barrier before and after the timed region and the maximum
of the per-rank times.  These helpers work with any torch.distributed backend (NCCL on the GPU
node, gloo in the CPU tests).
"""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


def world() -> tuple[int, int]:
    """(rank, world size) from the torchrun environment (0, 1 without it)."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def shard(n_items: int, rank: int, world_size: int) -> range:
    """Contiguous share of n_items for `rank`: sizes differ by at most one, earlier ranks larger."""
    base, extra = divmod(n_items, world_size)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def barrier():
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank float over all ranks (the value itself on one rank)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def job_throughput(units_this_rank: float, seconds_this_rank: float, device=None) -> float:
    """Whole-job rate: the units all ranks processed over the slowest rank's time."""
    return sum_over_ranks(units_this_rank, device) / max_over_ranks(seconds_this_rank, device)
