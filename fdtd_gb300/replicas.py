"""Replica bookkeeping for multi-GPU runs.

The FDTD step of one solve is not sharded across GPUs here: every GPU of a
node runs its own independent solve (weak scaling, no data-path collective).
The only cross-rank communication is timing: a barrier before and after the
timed region and a max-reduction of the elapsed time.
"""
from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(rank, local_rank, world_size) from the torchrun environment."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def barrier(dist) -> None:
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def aggregate(units: float, seconds: float, dist=None, device=None) -> tuple[float, float]:
    """Total units over ranks and the slowest rank's time."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(units), float(seconds)
    import torch

    t = torch.tensor([float(units), float(seconds)], dtype=torch.float64, device=device)
    u = t[:1].clone()
    s = t[1:].clone()
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    return float(u.item()), float(s.item())
