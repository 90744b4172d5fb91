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
