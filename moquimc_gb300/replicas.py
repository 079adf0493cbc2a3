"""Replicas across GPUs of one node: the transport shards by history with no exchange inside a step.

Histories are independent, so N GPUs run N independent replicas (one process per GPU, launched by
torchrun): each rank draws its own source vertices and transport seed, transports its histories
into its own tallies, and the only exchange is one sum of the FP64 tallies at the end (moqui has
no multi-GPU path; its per-GPU jobs are combined by hand).  The step time reported is the maximum
over ranks.
"""
from __future__ import annotations

import os

VERTEX_SEED_BASE = 3
TRANSPORT_SEED_BASE = 0x5EED0000


def world() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment; (1, 0, 0) without it."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seeds(rank: int) -> tuple[int, int]:
    """(vertex seed, transport seed base) of a rank: distinct streams per replica."""
    return VERTEX_SEED_BASE + 1000 * rank, TRANSPORT_SEED_BASE + 7919 * rank


def history_range(n_total: int, rank: int, world_size: int) -> tuple[int, int]:
    """Contiguous share of n_total histories for a rank (strong scaling of one job)."""
    per = n_total // world_size
    extra = n_total % world_size
    h0 = rank * per + min(rank, extra)
    return h0, h0 + per + (1 if rank < extra else 0)


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of a per-rank value (the step time) over all ranks."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_tallies(tally, device=None):
    """Sum a per-rank FP64 tally (numpy array or tensor) over all ranks; returns a new tensor (the
    input is not modified)."""
    import numpy as np
    import torch
    import torch.distributed as dist

    t = torch.from_numpy(np.array(tally, copy=True)) if isinstance(tally, np.ndarray) else tally.clone()
    if device is not None:
        t = t.to(device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t
