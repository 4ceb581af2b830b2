"""Multi-GPU runs as independent replicas (no collective on the data path).

A DNS-aided solve does not shard here (its FFT projection needs global
transposes that the reference never distributes), and serving streams are
independent solves, so N GPUs run N replicas.  The only collectives are on
the host side of a measurement: a barrier around the timed region and the
maximum of the per-rank times, from which the whole-job rate is computed.
"""
from __future__ import annotations

import os


def world():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def slowest(seconds: float, device=None) -> float:
    """Maximum of a per-rank duration over all ranks (identity without a
    process group)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, seconds: float, world_size: int) -> float:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    return units_per_rank * world_size / seconds
