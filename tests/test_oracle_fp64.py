"""The FP64 oracle's full-physics operators checked against each other on the
CPU (they have no reference counterpart, so they are pinned by their own
algebra): the least-squares pair ko_lsm_apply is adjoint in double
precision, and its migration L^T applied to a survey's traces gives the
accumulators of the full-mode job ko_kirchhoff64 of the same survey."""
from __future__ import annotations

import numpy as np
import pytest

from random_gb300 import capi, synth


def _survey(**kw):
    base = dict(ntr=240, ns=201, dt=0.004, nx=8, ny=6, bin_m=25.0, max_offset=900.0, n_refl=2, n_diff=6,
                freq=25.0, aperture=350.0, aa_cutoff=60.0, seed=31, mode=capi.MODE_FULL, output=capi.OUT_STACK)
    base.update(kw)
    return synth.patch3d(**base)


@pytest.mark.parametrize("output", [capi.OUT_STACK, capi.OUT_OFFSET_GATHERS])
def test_fp64_operator_pair_is_adjoint(oracle_lib, output):
    kw = dict(output=output) if output == capi.OUT_STACK else dict(output=output, nh=3, oh=0.0, dh=400.0)
    s = _survey(**kw)
    shape = capi.oracle_dims(s.params)["shape"]
    rng = np.random.default_rng(3)
    for _ in range(2):
        m = rng.normal(size=shape)
        d = rng.normal(size=(s.ntr, s.ns))
        lm = oracle_lib.lsm_apply(s, 1, m)
        ltd = oracle_lib.lsm_apply(s, 0, d)
        a, b = float((lm * d).sum()), float((m * ltd).sum())
        assert abs(a - b) <= 1e-12 * abs(a), (a, b)


def test_fp64_adjoint_is_the_full_mode_job(oracle_lib):
    s = _survey()
    km = oracle_lib.kirchhoff64(s)["km"]
    lt = oracle_lib.lsm_apply(s, 0, s.samples.astype(np.float64))
    assert np.linalg.norm(km) > 0
    assert np.linalg.norm(lt - km) <= 1e-6 * np.linalg.norm(km)
