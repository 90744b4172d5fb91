"""The CPU oracle is pinned to the reference: it must reproduce the golden
fixtures (made by the compiled reference) bit for bit, and - where the
reference checkout is present - fresh runs of the compiled reference on
random small configurations."""
from __future__ import annotations

import tempfile
from pathlib import Path

import numpy as np
import pytest

from fixtures import NAMES, load, rel_l2
from random_gb300 import segy, synth


def _oracle_job_images(oracle_lib, s, jx, jy):
    out = []
    for job in range(jx * jy):
        r = oracle_lib.kirchhoff(s, dict(jobs_x=jx, jobs_y=jy, job_id=job), want_acc=False)
        out.append(r["image"].reshape(-1, s.ns))
    return np.concatenate(out)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_golden_bit_exact(oracle_lib, name):
    s, jx, jy, image, _, _ = load(name)
    got = _oracle_job_images(oracle_lib, s, jx, jy)
    assert got.shape == image.shape
    assert np.array_equal(got.view(np.uint32), image.view(np.uint32)), rel_l2(got, image)


def test_golden_inputs_decode_like_reference():
    # the IBM words stored in the fixtures decode (reference formula) to the
    # samples the fixture survey uses
    s, _, _, _, _, ibm = load("g1_line_oddns")
    assert np.array_equal(segy.ibm_to_ieee(ibm), s.samples)
    assert np.array_equal(segy.ieee_to_ibm(s.samples), ibm)


def test_aliasfilter_odd_ns_quirk(oracle_lib):
    # Kirchhoff.c:419-423 zeroes bins ns/2 and ns/2+1 for odd ns
    tm, aa = oracle_lib.aliasfilter(1001, np.float32(0.004), 25.0, 25.0, 1e6)
    assert tm == 8
    assert aa[500] == 0.0 and aa[501] == 0.0
    assert np.all(aa[:500] == 1.0) and np.all(aa[502:] == 1.0)
    tm, aa = oracle_lib.aliasfilter(1000, np.float32(0.004), 25.0, 25.0, 40.0)
    assert aa[500] > 0 and np.allclose(aa[1:500], aa[:500:-1])


def test_prep_trace_mirror_and_tail(oracle_lib):
    ns, tm, dt = 50, 5, np.float32(0.004)
    t2 = np.array([np.float32(0.25 * t * t * float(dt) * float(dt)) for t in range(ns)], np.float32)
    f = np.random.default_rng(0).normal(size=ns).astype(np.float32)
    P = oracle_lib.prep_trace(f, t2, tm, float(dt))
    assert P.size == ns + 2 * tm
    for j in range(1, tm + 1):                    # mirror: P[-j] = P[j]
        assert P[tm - j] == P[tm + j]
    assert P[tm] == f[0]


from oracle.refbuild import REFERENCE_SOURCE  # noqa: E402  (the recipe owns the reference location)

ref_present = REFERENCE_SOURCE.exists()


@pytest.mark.skipif(not ref_present, reason="reference checkout absent")
@pytest.mark.parametrize("seed", [11, 12])
def test_oracle_matches_fresh_reference_runs(oracle_lib, seed):
    from oracle import refbuild
    rng = np.random.default_rng(seed)
    ns = int(rng.integers(120, 260))
    s = synth.patch3d(ntr=int(rng.integers(80, 200)), ns=ns, dt=0.004, nx=int(rng.integers(3, 7)),
                      ny=int(rng.integers(2, 6)), bin_m=25.0, max_offset=900.0, n_refl=2, n_diff=4,
                      freq=25.0, aperture=float(rng.uniform(150, 400)), aa_cutoff=float(rng.uniform(20, 90)),
                      seed=seed, mode=0, output=0, nh=3, oh=0.0, dh=250.0,
                      rotate_deg=float(rng.uniform(-40, 40)), origin=(1500.0, 900.0))
    jx, jy = int(rng.integers(1, 3)), int(rng.integers(1, 3))
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        s.write_files(td / "d.segy", td / "v.segy")
        b = refbuild.compile(refbuild.RefConfig(**s.ref_config(jobs_x=jx, jobs_y=jy)), tag="t")
        refbuild.run(b, td / "run", td / "d.segy", td / "v.segy", nprocs=jx * jy)
        _, ref = refbuild.read_image(td / "run", ns, jx * jy)
    got = _oracle_job_images(oracle_lib, s, jx, jy)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), rel_l2(got, ref)


def test_restatement_is_the_reference_on_the_full_line(oracle_lib):
    """The 2-D line at full size (200 CMPs x 48 offsets x 1001 samples, 1.61e9
    pairs): the C restatement's finished image has exactly the bytes of the
    compiled reference's own output (its SHA-256 recorded by
    tests/golden/make_golden.py)."""
    from fixtures import line2d_golden, image_sha256
    gold = line2d_golden()
    s = synth.line2d()
    o = oracle_lib.kirchhoff(s, want_acc=False)
    img = o["image"].reshape(-1, s.ns)
    assert img.shape == (gold["traces"], gold["ns"])
    assert image_sha256(img) == gold["sha256"]
    assert o["pairs"] > 1.5e9
