"""Multi-process host logic on CPU (gloo, world size 2): the reference's
round-robin job assignment, the per-rank slab parameters, the benchmark's
timing/pair reductions, and that slabs imaged independently reassemble the
whole image (checked with the oracle, as the GPU path is one slab per rank)."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from random_gb300 import multirank, synth


def test_round_robin_matches_reference_loop():
    # for (job = rank; job < no_job; job += size), Kirchhoff.c:347
    assert multirank.jobs_of(0, 3, 8) == [0, 3, 6]
    assert multirank.jobs_of(2, 3, 8) == [2, 5]
    every = sorted(j for r in range(4) for j in multirank.jobs_of(r, 4, 13))
    assert every == list(range(13))
    with pytest.raises(ValueError):
        multirank.jobs_of(3, 3, 8)


def test_slabs_reassemble_the_image(oracle_lib):
    s = synth.line2d(n_cmp=20, n_off=4, ns=151, seed=7)
    whole = oracle_lib.kirchhoff(s, want_acc=True)
    parts = []
    for rank in range(2):
        for p in multirank.slab_params(s.params, rank, 2):
            parts.append((p["job_id"], oracle_lib.kirchhoff(s, p, want_acc=True)))
    parts.sort(key=lambda x: x[0])
    km = np.concatenate([r["km"] for _, r in parts])
    assert np.array_equal(km, whole["km"])
    img = np.concatenate([r["image"] for _, r in parts])
    assert np.array_equal(img, whole["image"])


def _free_port() -> int:
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        elapsed = 1.0 + rank          # rank 1 is the slow one
        pairs = 1000 * (rank + 1)
        t, p = multirank.reduce_timing(elapsed, pairs)
        q.put((rank, t, p, [d["job_id"] for d in multirank.slab_params({}, rank, world, jobs_x=5)]))
    finally:
        dist.destroy_process_group()


def test_two_rank_reductions_over_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.0, 2.0]          # max over ranks
    assert [o[2] for o in out] == [3000.0, 3000.0]    # sum over ranks
    assert out[0][3] == [0, 2, 4] and out[1][3] == [1, 3]


def test_lsm_decomposition_choice():
    # the least-squares survey: 250,000 traces x 751 against a 200 x 200 x 751 model
    d = multirank.lsm_decomposition(250_000, 751, 200 * 200 * 751, 8)
    assert d["choice"] == "trace_shards" and d["trace_shards_bytes"] < d["image_slabs_bytes"] / 6
    assert multirank.lsm_decomposition(1000, 751, 200 * 200 * 751, 2)["choice"] == "image_slabs"
    assert multirank.lsm_decomposition(1000, 751, 10, 1)["trace_shards_bytes"] == 0.0
    sl = [multirank.trace_shard(10, r, 3) for r in range(3)]
    assert [(s.start, s.stop) for s in sl] == [(0, 4), (4, 8), (8, 10)]


def _lsm_survey():
    from random_gb300 import capi
    return synth.patch3d(ntr=160, ns=161, dt=0.004, nx=6, ny=5, bin_m=25.0, max_offset=900.0, n_refl=2, n_diff=4,
                         freq=25.0, aperture=350.0, aa_cutoff=60.0, seed=21, mode=capi.MODE_FULL,
                         output=capi.OUT_STACK)


def _lsm_data(s):
    from oracle import oracle
    rng = np.random.default_rng(3)
    m_true = np.zeros((6, 5, 1, s.ns))
    m_true[:, :, 0, 50] = 1.0
    m_true[2, 3, 0, 90] = -2.0
    d = oracle.lsm_apply(s, 1, m_true)
    return d + 0.05 * np.std(d) * rng.normal(size=d.shape)


def _lsm_worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    from oracle import oracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        s = _lsm_survey()
        d = _lsm_data(s)
        sl = multirank.trace_shard(s.ntr, rank, world)
        sub = synth.Survey(s.name, s.params, s.velocity, s.headers[sl], s.samples[sl])
        fwd = lambda m: torch.from_numpy(oracle.lsm_apply(sub, 1, m.numpy()))
        adj = lambda r: torch.from_numpy(oracle.lsm_apply(sub, 0, r.numpy()))
        x, res = multirank.cgls_trace_shards(fwd, adj, torch.from_numpy(d[sl]), 5)
        q.put((rank, x.numpy(), res))
    finally:
        dist.destroy_process_group()


def test_two_rank_trace_sharded_cgls_equals_one_rank(oracle_lib):
    """Two gloo ranks, each with half the traces and the FP64 oracle operators
    for them, run CGLS with one model all-reduce per iteration and reach the
    single-rank FP64 CGLS iterate (to summation-order rounding)."""
    import torch.multiprocessing as mp
    s = _lsm_survey()
    x1, res1 = oracle_lib.cgls(s, _lsm_data(s), 5)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_lsm_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in procs), key=lambda o: o[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, x, res in out:
        assert np.allclose(res, res1, rtol=1e-12, atol=0)
        assert np.linalg.norm(x - x1[-1]) <= 1e-12 * np.linalg.norm(x1[-1])
    assert np.array_equal(out[0][1], out[1][1])  # the replicated model is the same on every rank


def _slab_worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    from oracle import oracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        s = _lsm_survey()
        d = _lsm_data(s)
        sl = multirank.image_slab(6, rank, world)

        def fwd(m_slab):
            m = np.zeros((6, 5, 1, s.ns))
            m[sl] = m_slab.numpy()
            return torch.from_numpy(oracle.lsm_apply(s, 1, m))

        adj = lambda r: torch.from_numpy(np.ascontiguousarray(oracle.lsm_apply(s, 0, r.numpy())[sl]))
        x, res = multirank.cgls_image_slabs(fwd, adj, torch.from_numpy(d), 5)
        q.put((rank, x.numpy(), res))
    finally:
        dist.destroy_process_group()


def test_two_rank_image_slab_cgls_equals_one_rank(oracle_lib):
    """Two gloo ranks, each with half the inlines of the image (the
    reference's slabs) and the whole data, run CGLS with one data all-reduce
    per iteration; their slabs put together are the single-rank FP64 CGLS
    iterate (to summation-order rounding)."""
    import torch.multiprocessing as mp
    s = _lsm_survey()
    x1, res1 = oracle_lib.cgls(s, _lsm_data(s), 5)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_slab_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in procs), key=lambda o: o[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, _, res in out:
        assert np.allclose(res, res1, rtol=1e-12, atol=0)
    x = np.concatenate([o[1] for o in out], axis=0)
    assert x.shape == x1[-1].shape
    assert np.linalg.norm(x - x1[-1]) <= 1e-12 * np.linalg.norm(x1[-1])

