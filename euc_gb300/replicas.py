"""Replica scaling for the batched and serving forms.

Scenes are independent, so N GPUs run N replicas: every rank renders its own
seeded scenes (no collective on the data path).  The only exchange is on the
host side of the measurement: the slowest rank's step time, and the whole
job's rate over that time.  torch.distributed is plumbing here (NCCL on GPUs,
gloo on CPU in the tests).
"""
import os


def dist_env():
    """(world size, rank, local rank) from the torchrun environment."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_seed(seed, rank):
    """Seed of a rank's scenes: ranks render different, reproducible scenes."""
    return seed + 1000 * rank


def max_over_ranks(value, device=None):
    """The largest `value` (a float) over all ranks; `value` itself when the
    process group is not initialised (one replica)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device=None):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds_max):
    """Units of all ranks per second of the slowest rank (weak scaling)."""
    return world * units_per_rank / seconds_max
