"""Multi-GPU helpers: replicas, particle shards and their reductions.

The path shards without any collective on its data: candidates are
independent, and particles are independent up to one float64 partial sum
per candidate (the reference shards by STAR line range and concatenates its
text output, R/wrap_to_search_v2.py:83-101). One process per GPU scores its
own candidates (replicas) or its own particle range (shards); the host-side
reductions below are the only exchange: the maximum of per-rank times for a
job-wide rate, and the float64 sum of per-shard scores. They run on any
torch.distributed backend (NCCL between GPUs, gloo on CPU for the tests).
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

__all__ = ["replica_seed", "particle_shard", "max_over_ranks", "sum_over_ranks", "job_rate"]


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of a replica's synthetic candidates: distinct per rank."""
    return int(base_seed) + 7919 * int(rank)


def particle_shard(n_particles: int, world: int, rank: int) -> Tuple[int, int]:
    """[begin, end) of the contiguous particle range of ``rank`` (sizes differ by at most one)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    q, r = divmod(int(n_particles), int(world))
    begin = rank * q + min(rank, r)
    return begin, begin + q + (1 if rank < r else 0)


def _reduce(values: Sequence[float], op, device) -> List[float]:
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=op)
    return [float(x) for x in t.cpu()]


def max_over_ranks(values: Sequence[float], device="cpu") -> List[float]:
    """Element-wise maximum over ranks (times of the slowest rank)."""
    import torch.distributed as dist
    return _reduce(values, dist.ReduceOp.MAX, device)


def sum_over_ranks(values: Sequence[float], device="cpu") -> List[float]:
    """Element-wise float64 sum over ranks (per-candidate scores of particle shards)."""
    import torch.distributed as dist
    return _reduce(values, dist.ReduceOp.SUM, device)


def job_rate(world: int, units_per_rank: float, max_elapsed_s: float) -> float:
    """Job-wide units per second: every rank's units over the slowest rank's time."""
    return world * units_per_rank / max_elapsed_s if max_elapsed_s > 0 else 0.0
