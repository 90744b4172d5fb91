"""Precision mode (KPSTM_PREC_BF16_KAHAN): traces stored as bf16 with a
per-trace power-of-two scale, tap tables built from them with double
integrals, fp32 traveltimes, Kahan-compensated accumulation.  Errors are
measured against the FP64 oracle (every quantity in double).

Two workloads: the 2-D line at full size (200 CMPs x 48 offsets x 1001
samples, reference operator) and a 64 x 64 x 1501 sub-volume of the 3-D
generator (full physics).  Measured on a GB300 (relative L2 / peak):
  line, fp32 reference arithmetic   image 0.49  (the reference's own float
                                    running integrals of f/t^2; the
                                    compiled reference shows the same)
  line, bf16 + Kahan                image 4.2e-3, km 3.5e-3
  sub-volume, fp32                  image 1.9e-4
  sub-volume, bf16 + Kahan          image 9.8e-4, peak 3.3e-3
The bars below are those with margin."""
from __future__ import annotations

import numpy as np
import pytest

from fixtures import rel_l2
from random_gb300 import capi, synth
from random_gb300.migration import migrate

pytestmark = pytest.mark.gpu


def _peak(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_line_bf16_kahan_vs_fp64(kpstm_lib, oracle_lib):
    s = synth.line2d()
    o = oracle_lib.kirchhoff64(s)
    g16 = migrate(s, dict(precision=capi.PREC_BF16_KAHAN), want_acc=True)
    g32 = migrate(s, want_acc=True)
    e16, e32 = rel_l2(g16["image"], o["image"]), rel_l2(g32["image"], o["image"])
    assert e16 <= 1e-2, e16
    assert rel_l2(g16["km"], o["km"]) <= 1e-2
    assert e16 < 0.1 * e32, (e16, e32)  # far closer to exact than the reference's float integrals
    assert np.mean(g16["fold"] == o["fold"]) >= 0.9999


def test_subvolume_bf16_kahan_vs_fp64(kpstm_lib, oracle_lib):
    s = synth.patch3d(ntr=400, ns=1501, dt=0.002, nx=64, ny=64, bin_m=25.0, max_offset=4000.0, n_refl=8,
                      n_diff=40, freq=30.0, aperture=3000.0, aa_cutoff=100.0, seed=2, mode=capi.MODE_FULL,
                      output=capi.OUT_STACK)
    o = oracle_lib.kirchhoff64(s)
    g32 = migrate(s, want_acc=True)
    g16 = migrate(s, dict(precision=capi.PREC_BF16_KAHAN), want_acc=True)
    assert rel_l2(g32["image"], o["image"]) <= 1e-3
    e16 = rel_l2(g16["image"], o["image"])
    assert e16 <= 3e-3, e16
    assert _peak(g16["image"], o["image"]) <= 1e-2
    assert rel_l2(g16["km"], o["km"]) <= 3e-3
