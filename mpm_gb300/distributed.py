"""Multi-rank runs: one process per GPU, no collective on the data path.

A single scene does not shard (the quadratic stencil needs a 2-cell halo exchange and particle
migration, which the reference does not have either), so N ranks run N replicas.  Batched
independent scenes shard by scene: rank r takes scenes r, r + N, r + 2N, ...  The only
collectives are the timing ones: a barrier around the timed region and the maximum of the
ranks' times, so that a whole-job rate is (units of all ranks) / (slowest rank's time).
"""
from __future__ import annotations

import os


def env():
    """(world, rank, local_rank) from the torchrun environment (1, 0, 0 when absent)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str | None = None):
    """Initialise the default process group when world > 1 (nccl on GPUs, gloo otherwise)."""
    import torch
    import torch.distributed as dist

    world, rank, local = env()
    if world > 1 and not dist.is_initialized():
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def shard(items, rank: int, world: int):
    """Rank `rank`'s share of independent work items: items rank, rank + world, ..."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError(f"rank {rank} outside world {world}")
    return items[rank::world]


def barrier():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(value: float) -> float:
    """The largest of the ranks' values (the value itself on one rank)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def job_rate(units_all_ranks: float, seconds_slowest: float) -> float:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    if not seconds_slowest > 0:
        raise ValueError("time must be positive")
    return float(units_all_ranks) / float(seconds_slowest)
