"""Replica bookkeeping for multi-GPU runs.

The solve path has no data-parallel split (one context, one GPU); with N
GPUs every rank solves its own replica (independent load cases or designs)
and the job reports the slowest rank's time.  These helpers wrap the
torch.distributed calls so that the same code runs on NCCL (GPU ranks) and
on gloo (the CPU tests).
"""
from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str, timeout_s: float | None = None) -> None:
    """Joins the process group.  A rank that dies or stops between steps must not
    leave the others waiting forever in their next collective: the group's
    timeout (`timeout_s`, else SGLD_PG_TIMEOUT_S, else 600 s) bounds every wait,
    after which the waiting ranks' collective raises.  (A peer whose process has
    exited usually ends the wait sooner: its connections close.)"""
    import datetime

    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    rank, world, _ = dist_env()
    if world > 1 and not dist.is_initialized():
        if timeout_s is None:
            timeout_s = float(os.environ.get("SGLD_PG_TIMEOUT_S", "600"))
        dist.init_process_group(backend, rank=rank, world_size=world,
                                timeout=datetime.timedelta(seconds=timeout_s))


def barrier() -> None:
    import torch.distributed as dist

    if dist.is_initialized():
        dist.barrier()


def aggregate(seconds: float, units: float, device=None) -> tuple[float, float]:
    """(max over ranks of `seconds`, sum over ranks of `units`)."""
    import torch
    import torch.distributed as dist

    if not dist.is_initialized():
        return float(seconds), float(units)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def shutdown() -> None:
    import torch.distributed as dist

    if dist.is_initialized():
        dist.destroy_process_group()
