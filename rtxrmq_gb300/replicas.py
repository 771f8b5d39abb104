"""Replicas across GPUs: one process per GPU (torchrun), one index per GPU.

Range-minimum queries are independent, and every GPU holds its own copy of the
index, so a multi-GPU run is N replicas with no collective on the data path:
each rank answers its own query set. A multi-rank benchmark needs three host
pieces, kept here so that they run (and are tested) without a GPU:

* the rank's query-set seed (different per rank, fixed per rank and mode),
* the step time as the maximum over ranks (a collective on the timing only),
* the whole-job rate: every rank's queries over that time.
"""
from __future__ import annotations


def rank_seed(base: int, rank: int, lr: int) -> int:
    """Seed of rank `rank`'s query set for length mode `lr`."""
    return base + 1 + 1000 * rank + (0 if lr == -1 else 17 * abs(lr))


def world() -> tuple[int, int]:
    """(rank, world size) of the initialised process group, else (0, 1)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def max_over_ranks(x: float, device=None) -> float:
    """Maximum of `x` over the ranks of the process group (x itself on one
    rank). `device`: where the reduction buffer lives (a CUDA device under
    NCCL, None (CPU) under gloo)."""
    import torch
    import torch.distributed as dist
    if world()[1] == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: int, n_ranks: int, ms_per_step: float) -> float:
    """Whole-job throughput: all ranks' units per step over the (max-over-
    ranks) step time in milliseconds."""
    return n_ranks * units_per_rank / (ms_per_step / 1e3)
