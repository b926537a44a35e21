"""Multi-GPU runs of the search: the sky partitioned over the GPUs.

Sky points are independent and the search has no exchange step, so N GPUs
split the sky as the reference splits it over processes with -range files
(search/network/src-cpu/init.c:664-700): each rank (one process per GPU,
its own context and copy of the detector data) takes a contiguous block of
sky points in the sky loop's order (contiguous mm ranges), and the only
communication is the benchmark's timing reduction: the step time is the
maximum over ranks and the work the sum over ranks.  torch.distributed
carries it (NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

import os


def world() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", os.environ.get("RANK", "0"))))


def init(backend: str | None = None) -> bool:
    """Initialises the default process group when WORLD_SIZE > 1 (rendezvous
    from MASTER_ADDR / MASTER_PORT).  Returns True when one was created."""
    import torch
    import torch.distributed as dist
    rank, size, _ = world()
    if size <= 1 or dist.is_initialized():
        return False
    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend, rank=rank, world_size=size)
    return True


def shard(tasks: list, rank: int, size: int, per_rank: int | None = None) -> list:
    """The rank's contiguous block of the sky points `tasks` (in sky-loop
    order): blocks of `per_rank` points (default: len(tasks) // size, the
    last rank taking the remainder); blocks of different ranks are
    disjoint."""
    if size <= 1:
        return list(tasks if per_rank is None else tasks[:per_rank])
    if per_rank is None:
        per = len(tasks) // size
        lo = rank * per
        hi = len(tasks) if rank == size - 1 else lo + per
        return list(tasks[lo:hi])
    return list(tasks[rank * per_rank:(rank + 1) * per_rank])


def barrier() -> None:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def reduce_step(seconds: float, units: float) -> tuple[float, float]:
    """(max of `seconds` over ranks, sum of `units` over ranks); the local
    values when no process group is up."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return seconds, units
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([seconds], dtype=torch.float64, device=dev)
    u = torch.tensor([units], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def shutdown() -> None:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
