"""Multi-process host logic: one process per GPU, each imaging its own slab.

The reference partitions the image box into independent slabs
(number_mpi_jobsX x number_mpi_jobsY, Kirchhoff.c:64-65, 280-300) and deals
them out round-robin, ``for (job = rank; job < no_job; job += size)``
(Kirchhoff.c:347); every slab reads all traces and no data is exchanged.
Here a rank owns the jobs the same loop would give it and runs them on its
GPU; the only collectives are the timing and pair-count reductions of the
benchmark (max of elapsed times, sum of pairs), which work over gloo or
nccl alike.
"""
from __future__ import annotations


def jobs_of(rank: int, world: int, no_job: int) -> list[int]:
    """The reference's round-robin job loop (Kirchhoff.c:347)."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    return list(range(rank, no_job, world))


def slab_params(params: dict, rank: int, world: int, jobs_x: int | None = None, jobs_y: int = 1) -> list[dict]:
    """kpstm_params overrides for each job (slab) this rank images when the
    image box is cut into jobs_x * jobs_y slabs (default: one slab per rank
    along x)."""
    jx = world if jobs_x is None else jobs_x
    return [dict(params, jobs_x=jx, jobs_y=jobs_y, job_id=j) for j in jobs_of(rank, world, jx * jobs_y)]


def weak_scaling_shift(rank: int, width_m: float) -> float:
    """x offset of rank's own survey region when every rank images a
    full-size slab of a wider survey (fixed work per GPU)."""
    return rank * width_m


def reduce_timing(elapsed_s: float, pairs: float, device=None) -> tuple[float, float]:
    """(max elapsed over ranks, total pairs) via torch.distributed; identity
    when no process group is initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(elapsed_s), float(pairs)
    t = torch.tensor([float(elapsed_s)], dtype=torch.float64, device=device)
    p = torch.tensor([float(pairs)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(p, op=dist.ReduceOp.SUM)
    return float(t.item()), float(p.item())
