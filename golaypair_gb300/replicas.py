"""Replicas on several GPUs: one process per GPU, no data-path collective.

The search shards by word-rank ranges (the reference's `-j/-n` job split,
src/utils/lyndon.cpp:93-106, via `job_ranges`): each replica runs its own
jobs, and replicas meet only to agree on a time (the maximum over ranks) and
to add up counts.  These helpers take whatever torch.distributed backend the
process group was created with (NCCL on GPUs, gloo in the CPU tests).
"""
import os


def dist_env():
    """(world_size, rank, local_rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _reduce(value, op, device):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value, device=None):
    """The largest of every rank's value (the job's time is the slowest
    replica's)."""
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.MAX, device)


def sum_over_ranks(value, device=None):
    """The sum of every rank's value (units processed by all replicas)."""
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.SUM, device)


def jobs_of_rank(rank, world_size, njobs):
    """The jobs (of a `-n njobs` split) replica `rank` of `world_size` runs:
    rank, rank + world_size, ..."""
    return list(range(rank, njobs, world_size))
