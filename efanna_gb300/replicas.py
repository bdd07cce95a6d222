"""Replicas across GPUs of one node: one process per GPU, each holding the whole index.

The search does not shard its data path (queries are independent; the build's join/update scatter
into arbitrary nodes and would need an all-to-all per iteration), so ranks never exchange search
data: they meet only to start and stop the same timed steps, and the slowest rank's time counts.
Launch with torch.distributed.run (RANK / WORLD_SIZE / LOCAL_RANK / MASTER_ADDR / MASTER_PORT in
the environment); the rendezvous address defaults to 127.0.0.1.
"""
from __future__ import annotations

import os


def world():
    """(world size, rank, local rank) from the launcher's environment (1, 0, 0 without one)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str = "nccl") -> bool:
    """Joins the process group when there are several ranks; True if it did."""
    ws, _, local = world()
    if ws <= 1:
        return False
    import torch
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return True


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(value: float, device=None) -> float:
    """The largest `value` over all ranks (the slowest rank's time)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def throughput(units_per_rank: float, seconds_max: float, world_size: int) -> float:
    """Whole-job units per second: every rank's units over the slowest rank's time."""
    return world_size * units_per_rank / seconds_max


def query_slice(nq: int, rank: int, world_size: int):
    """Contiguous share [start, stop) of nq queries for a rank (shares differ by at most one)."""
    base, extra = divmod(nq, world_size)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def finish():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
