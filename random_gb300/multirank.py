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


# ------------------------------------------------------------------ LSM
# Least-squares migration couples the slabs: L m sums every slab's
# contribution into every trace.  Two decompositions, per CG iteration:
#   image slabs  - L p needs a data-space all-reduce (ntr x ns floats), L^T r
#                  runs per slab on the replicated residual;
#   trace shards - L p runs per shard on the replicated search direction,
#                  L^T r needs a model-space all-reduce (nx x ny x nh x ns).
# Both also reduce two FP64 scalars per iteration.  lsm_decomposition picks
# the smaller all-reduce; for the 250,000-trace, 200 x 200 x 751 least-squares
# survey that is the trace shards (120 MB per iteration instead of 751 MB).


def lsm_decomposition(ntr: int, ns: int, model_elems: int, world: int) -> dict:
    """Bytes one rank sends per CG iteration (ring all-reduce: 2 (N-1)/N of
    the vector) for each decomposition, and the choice."""
    f = 2.0 * (world - 1) / world if world > 1 else 0.0
    slab = f * 4.0 * ntr * ns
    shard = f * 4.0 * model_elems
    return {"image_slabs_bytes": slab, "trace_shards_bytes": shard,
            "choice": "trace_shards" if shard <= slab else "image_slabs"}


def trace_shard(ntr: int, rank: int, world: int) -> slice:
    """Contiguous block of traces of one rank (block order is kept, so the
    shards concatenate to the survey)."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    per = -(-ntr // world)
    return slice(min(ntr, rank * per), min(ntr, (rank + 1) * per))


def image_slab(nx: int, rank: int, world: int) -> slice:
    """Contiguous block of inlines (image columns in x) of one rank: the
    reference's slabs along x (Kirchhoff.c:280-300)."""
    return trace_shard(nx, rank, world)


def _allreduce(t):
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t


def _dot(x, y) -> float:
    """FP64 dot product of two tensors, summed over the ranks."""
    import torch
    v = torch.sum(x.double() * y.double()).reshape(1)
    return float(_allreduce(v).item())


def cgls_trace_shards(forward, adjoint, d_local, niter: int, store=None):
    """CGLS on min |L m - d|^2 from m = 0 with the traces split across the
    ranks (the recurrence of kpstm_lsm_cg, including skipping the last
    search direction).  Each rank passes its own traces' data d_local and
    operators for them: forward(model) -> local data, adjoint(local data) ->
    its partial image.  Model-space vectors are replicated: the partial
    images are summed by one all-reduce per iteration, the data-space dot
    products by scalar all-reduces, and every rank takes the same FP64 step
    lengths.  ``store`` (optional) rounds the local residual as the storage
    format would (e.g. bf16 with a per-trace scale).  Returns (model,
    residual norms [niter + 1])."""
    import torch
    store = store or (lambda v: v)
    r = store(d_local.clone())
    res = [_dot(r, r) ** 0.5]
    s = _allreduce(adjoint(r))
    x = torch.zeros_like(s)
    if niter == 0:
        return x, res
    p = s.clone()
    gamma = float(torch.sum(s.double() * s.double()))
    for it in range(niter):
        q = forward(p)
        qq = _dot(q, q)
        alpha = gamma / qq if qq > 0 else 0.0
        x.add_(p, alpha=alpha)
        r = store(r.sub_(q, alpha=alpha))
        res.append(_dot(r, r) ** 0.5)
        if it + 1 == niter:
            break
        s = _allreduce(adjoint(r))
        gnew = float(torch.sum(s.double() * s.double()))
        p = s.add_(p, alpha=gnew / gamma if gamma > 0 else 0.0)
        gamma = gnew
    return x, res


def _local_dot(x, y) -> float:
    """FP64 dot product of two replicated tensors (no exchange)."""
    import torch
    return float(torch.sum(x.double() * y.double()))


def cgls_image_slabs(forward, adjoint, d, niter: int, store=None):
    """CGLS on min |L m - d|^2 from m = 0 with the image cut into slabs across
    the ranks (the reference's decomposition, Kirchhoff.c:280-300) and the
    same recurrence as cgls_trace_shards.  Each rank holds its slab of every
    model-space vector and the whole data space, replicated: forward(model
    slab) -> that slab's contribution to every trace, summed over the ranks
    by one data all-reduce per iteration; adjoint(data) -> its slab's image,
    with no exchange.  Model-space dot products are summed by scalar
    all-reduces, data-space ones are local, and every rank takes the same FP64
    step lengths.  Returns (this rank's model slab, residual norms
    [niter + 1])."""
    import torch
    store = store or (lambda v: v)
    r = store(d.clone())
    res = [_local_dot(r, r) ** 0.5]
    s = adjoint(r)
    x = torch.zeros_like(s)
    if niter == 0:
        return x, res
    p = s.clone()
    gamma = _dot(s, s)
    for it in range(niter):
        q = _allreduce(forward(p))
        qq = _local_dot(q, q)
        alpha = gamma / qq if qq > 0 else 0.0
        x.add_(p, alpha=alpha)
        r = store(r.sub_(q, alpha=alpha))
        res.append(_local_dot(r, r) ** 0.5)
        if it + 1 == niter:
            break
        s = adjoint(r)
        gnew = _dot(s, s)
        p = s.add_(p, alpha=gnew / gamma if gamma > 0 else 0.0)
        gamma = gnew
    return x, res
