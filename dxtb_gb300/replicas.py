"""Several GPUs: independent replicas over molecule shards.

Single points of different molecules share nothing, so with one process per
GPU every rank solves its own molecules (its shard of the workload) and no
collective touches the data path.  The only exchanges are the host-side
barrier around a timed region and the maximum of the ranks' times, which is
what a whole-job rate is measured against (the slowest rank ends the job).
The reference has no multi-GPU path; its batched calculator
(``scf/unrolling/default.py:142-401``) is the single-process equivalent.
"""
from __future__ import annotations

from . import molgen


def batch_shard(rank: int, count: int = 512) -> list:
    """The molecules of ``rank``: its own ``count`` seeded 10-120-atom
    molecules (rank 0 gets the workload's first shard)."""
    return molgen.c2_batch(count, shard=rank)


def max_over_ranks(x: float, world: int, device=None) -> float:
    """Maximum of ``x`` over all ranks of the default process group."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(per_rank: int, world: int, steps: int, seconds: float) -> float:
    """Molecules per second of the whole job: every rank's molecules over
    the slowest rank's time."""
    if seconds <= 0:
        raise ValueError("non-positive time")
    return per_rank * world * steps / seconds
