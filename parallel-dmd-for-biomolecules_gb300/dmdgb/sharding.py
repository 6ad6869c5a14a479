"""Replica sharding over several GPUs of one node (one process per GPU).

Independent systems need no exchange: every rank advances its own replicas
(weak scaling: the per-rank workload is fixed) or its share of a fixed set
(strong scaling), and the only collective is the max-over-ranks of the step
time.  A single system is never split across GPUs (its events are causally
coupled).  The reference has no counterpart: it runs one system per MPI job.
"""
from __future__ import annotations

from typing import List


def replica_seed(rank: int, base: int = 1) -> int:
    """Seed of a rank's replica set for weak scaling (distinct per rank)."""
    return base + 1000 * rank


def shard(n_total: int, world: int, rank: int) -> List[int]:
    """Indices of a fixed set of n_total systems assigned to `rank` (strong
    scaling): round-robin, so sizes drawn in sequence spread evenly."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    return list(range(rank, n_total, world))


def max_over_ranks(value: float, device: str = "cpu") -> float:
    """The maximum of a per-rank value over the process group (the step time
    that counts is the slowest rank's); the value itself outside a group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
