"""Replica bookkeeping for runs on several GPUs of one node.

The direct sums have no exchange step between GPUs here: each rank advances its own
independent replica (or its own ensemble instances), so the only cross-rank operations are a
barrier around the timed region and the maximum of the ranks' times.  The whole-job rate is
the work of all ranks divided by that maximum (weak scaling)."""
from __future__ import annotations


def max_over_ranks(value: float, dist=None, device: str = "cpu") -> float:
    """The largest `value` over the ranks of the default process group (the value itself when
    there is no group).  `device` is where the reduction tensor lives: "cuda" for NCCL,
    "cpu" for gloo."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(work_per_rank: float, seconds: float, dist=None, device: str = "cpu") -> float:
    """Whole-job rate: (work per rank x world size) / (the slowest rank's seconds)."""
    world = dist.get_world_size() if dist is not None and dist.is_initialized() else 1
    return world * work_per_rank / max_over_ranks(seconds, dist, device)
