"""Multi-GPU form of the path: independent replicas, no data-path collective.

The transform and RI-K of one molecule never exchange data between GPUs, and a
batch of molecules splits into independent molecules.  Each rank therefore
runs its own replica (or its own share of a batch).  The only cross-rank steps
are host-side bookkeeping:

* ``shard``: round-robin assignment of independent units (molecules) to ranks;
* ``max_over_ranks``: the step time of the job is the slowest rank's;
* ``job_throughput``: units of all ranks divided by that time.

They work on any ``torch.distributed`` backend (NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations

from typing import List, Sequence, TypeVar

T = TypeVar("T")


def shard(items: Sequence[T], rank: int, world: int) -> List[T]:
    """This rank's share of independent units: items rank, rank + world, ..."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    return list(items[rank::world])


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank scalar over the default process group (identity without one)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: Sequence[float], max_seconds: float) -> float:
    """Whole-job rate: the units every rank processed over the slowest rank's time."""
    if max_seconds <= 0:
        raise ValueError("time must be positive")
    return float(sum(units_per_rank)) / max_seconds
