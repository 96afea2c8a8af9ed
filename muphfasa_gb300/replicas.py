"""Multi-GPU execution of the step: replicas only.

The step of one domain does not shard across GPUs in this build (one domain
per GPU; the reference's only cross-rank exchange is the FillBoundary halo of
a decomposed domain).  N ranks therefore advance N independent domains, one
per GPU, with no collective on the data path; the host-side helpers below
only synchronise the timed region and combine the per-rank timings
(max over ranks) and work (sum over ranks).
"""
from __future__ import annotations

import os


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str | None = None):
    """Initialises torch.distributed when launched with more than one rank."""
    rank, world, _ = rank_info()
    if world <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend or "nccl", rank=rank, world_size=world)
    return dist


def _tensor(x, device):
    import torch
    return torch.tensor([float(x)], dtype=torch.float64, device=device)


def barrier(dist, device=None):
    if dist is not None:
        if device is not None and dist.get_backend() == "nccl":
            dist.barrier(device_ids=[device.index if hasattr(device, "index") else int(device)])
        else:
            dist.barrier()


def max_over_ranks(dist, x: float, device="cpu") -> float:
    if dist is None:
        return float(x)
    t = _tensor(x, device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, x: float, device="cpu") -> float:
    if dist is None:
        return float(x)
    t = _tensor(x, device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
