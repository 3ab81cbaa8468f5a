"""Independent replicas on several GPUs (one process per GPU).

A multigrid solve does not shard across GPUs here: each rank solves its own
copy of the workload and nothing crosses GPUs on the data path.  The only
multi-rank steps are a barrier around the timed region and a MAX reduction of
the elapsed time, so the job's throughput is (units on all ranks) / (slowest
rank's time).
"""
from __future__ import annotations

import os


def world():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str | None = None):
    """Joins the process group when world_size > 1; returns torch.distributed or None."""
    n, _, _ = world()
    if n <= 1:
        return None
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))
    return dist


def barrier(dist) -> None:
    if dist is not None:
        dist.barrier()


def job_throughput(units_per_rank: float, elapsed_s: float, dist, device: str = "cpu"):
    """(units on all ranks / slowest rank's time, slowest time)."""
    if dist is None:
        return units_per_rank / elapsed_s, elapsed_s
    import torch
    t = torch.tensor([elapsed_s, units_per_rank], dtype=torch.float64, device=device)
    tmax = t[:1].clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    units = t[1:].clone()
    dist.all_reduce(units, op=dist.ReduceOp.SUM)
    return float(units.item()) / float(tmax.item()), float(tmax.item())
