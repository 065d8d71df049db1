"""Multi-GPU runs as independent replicas (one process per GPU).

Independent grids need no exchange, so N GPUs run N replicas of the workload
and the job's throughput is the total work over the slowest rank's time.
These helpers hold that logic; they work with any torch.distributed backend
(NCCL on GPUs, gloo on CPU for tests).
"""
import os

__all__ = ["dist_info", "max_over_ranks", "job_throughput"]


def dist_info():
    """(world_size, rank, local_rank) from the torchrun environment (1, 0, 0 if unset)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(value, device=None):
    """The maximum of a float over all ranks (the value itself without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, slowest_seconds):
    """Total units of all replicas over the slowest rank's time (weak scaling)."""
    if slowest_seconds <= 0:
        raise ValueError("time must be positive")
    return units_per_rank * world / slowest_seconds
