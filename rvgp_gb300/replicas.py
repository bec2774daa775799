"""Process-per-GPU replicas of the RVGP pipeline.

The reference runs one pipeline per process on the CPU and has no
distributed code.  Its work does not shard across GPUs without a halo
exchange in every sparse product, so several GPUs run independent replicas:
rank r builds its own seeded manifold, fits and predicts it, and the job's
time is the slowest rank's.  The only cross-rank operations are a barrier
before and after the timed region and one max-reduction of the measured
time, none of them on the data path.
"""
from __future__ import annotations

import os


def world():
    """(rank, world_size, local_rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of rank ``rank``'s synthetic inputs: every replica gets its own
    manifold sample, so no two ranks repeat the same work."""
    return int(base_seed) * 1_000_003 + int(rank)


def max_over_ranks(value: float, device=None) -> float:
    """Largest ``value`` over all ranks of the initialised process group
    (identity when torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(step_seconds: float, world_size: int) -> float:
    """Pipelines per second of the whole job: every rank finishes one pipeline
    per step, and a step lasts as long as its slowest rank."""
    return world_size / step_seconds
