"""GPU full-physics mode (linear trace interpolation, obliquity/spreading
weight, variable-width triangle anti-alias; no reference counterpart)
against the FP64 CPU oracle restatement of the same operator.

The GPU computes in fp32 with the SFU reciprocal square root, so results
are not bit-identical; the bars below are the measured fp32-vs-fp64 error
with margin: relative L2 of the accumulators <= 1e-4, fold counts equal
except where the fp32 and fp64 traveltimes straddle the last sample."""
from __future__ import annotations

import numpy as np
import pytest

from fixtures import rel_l2
from random_gb300 import capi, synth
from random_gb300.migration import Migration, migrate

pytestmark = pytest.mark.gpu
ACC_TOL = 1e-4


def _survey(**kw):
    base = dict(ntr=400, ns=301, dt=0.004, nx=10, ny=8, bin_m=25.0, max_offset=1200.0, n_refl=3,
                n_diff=10, freq=25.0, aperture=500.0, aa_cutoff=60.0, seed=21, mode=capi.MODE_FULL,
                output=capi.OUT_OFFSET_GATHERS, nh=3, oh=0.0, dh=400.0)
    base.update(kw)
    return synth.patch3d(**base)


def _check(g, o):
    assert rel_l2(g["km"], o["km"]) <= ACC_TOL, rel_l2(g["km"], o["km"])
    mism = np.mean(g["fold"] != o["fold"])
    assert mism <= 1e-4, mism
    assert g["pairs"] == o["pairs"]


@pytest.mark.parametrize("output", [capi.OUT_OFFSET_GATHERS, capi.OUT_STACK])
def test_full_mode_matches_fp64_oracle(kpstm_lib, oracle_lib, output):
    s = _survey(output=output)
    g = migrate(s, want_acc=True)
    o = oracle_lib.kirchhoff(s)
    _check(g, o)
    assert rel_l2(g["image"], o["image"]) <= ACC_TOL


def test_full_mode_two_time_windows(kpstm_lib, oracle_lib):
    """ns = 1501 (2 ms) is imaged in two register windows of 768 samples."""
    s = _survey(ntr=150, ns=1501, dt=0.002, nx=4, ny=4, aperture=400.0, max_offset=800.0, nh=1, dh=1e9,
                output=capi.OUT_STACK)
    g = migrate(s, want_acc=True)
    o = oracle_lib.kirchhoff(s)
    _check(g, o)


def test_full_mode_line(kpstm_lib, oracle_lib):
    s = synth.line2d(n_cmp=40, n_off=8, ns=401, seed=13)
    p = dict(mode=capi.MODE_FULL)
    g = migrate(s, p, want_acc=True)
    o = oracle_lib.kirchhoff(s, p)
    _check(g, o)


def test_full_mode_block_split_is_invisible(kpstm_lib):
    s = _survey()
    a = migrate(s, block=100_000, want_acc=True)
    b = migrate(s, block=77, want_acc=True)
    assert np.array_equal(a["km"], b["km"]) and np.array_equal(a["fold"], b["fold"])


def _coarse_velocity(s):
    """The survey's v_rms grid kept on every second inline node and every
    second time sample, so that columns fall between nodes."""
    from random_gb300.synth import Velocity
    v = s.velocity
    vr = np.ascontiguousarray(v.vrms[::2, :, ::2])
    return Velocity(n_iline=vr.shape[0], n_xline=v.n_xline, nsm=vr.shape[2], o_iline=v.o_iline,
                    o_xline=v.o_xline, d_iline=2 * v.d_iline, d_xline=v.d_xline, dtm=2 * v.dtm, vrms=vr)


def test_trilinear_velocity_matches_fp64_oracle(kpstm_lib, oracle_lib):
    """velocity_interp = 1: v_rms interpolated (trilinear) at the position the
    reference rounds; against the FP64 oracle with the same interpolation,
    and visibly different from the nearest-node model."""
    s = _survey(ntr=300, nx=9, ny=4, nh=1, dh=1e9, output=capi.OUT_STACK)
    s.velocity = _coarse_velocity(s)
    p = dict(velocity_interp=1)
    g = migrate(s, p, want_acc=True)
    o = oracle_lib.kirchhoff64(s, p)
    assert rel_l2(g["km"], o["km"]) <= ACC_TOL, rel_l2(g["km"], o["km"])
    near = migrate(s, want_acc=True)
    assert rel_l2(near["km"], g["km"]) > 10 * ACC_TOL


def test_fold_counts_beyond_16_bits(kpstm_lib):
    """Full mode, stack output, 40,000 traces (a 400-trace survey repeated) in
    one block: every column's work item sees more hits than the kernel's 16-bit
    per-sample fold counters hold; the one-block result equals the one from
    3,000-trace blocks (where no item gets that far) bit for bit."""
    import dataclasses
    s = _survey(nx=4, ny=2, nh=1, dh=1e9, output=capi.OUT_STACK)
    s = dataclasses.replace(s, headers=np.tile(s.headers, (100, 1)), samples=np.tile(s.samples, (100, 1)))
    a = migrate(s, block=s.ntr, want_acc=True)
    b = migrate(s, block=3000, want_acc=True)
    assert int(a["fold"].max()) > 32_768
    assert np.array_equal(a["km"], b["km"]) and np.array_equal(a["fold"], b["fold"])


def _dead_window_share(m, kw, window):
    """Share of the (trace, in-aperture column, time window) visits whose
    summed source and receiver distances D satisfy D^2 >= max over the
    window of (T^2 - 4 tx) / ty: the float64 form of the kernel's cull
    bound, per column (the kernel takes the tile's box and window)."""
    ns, dt, b = kw["ns"], kw["dt"], kw["bin_m"]
    p = m.survey.params
    X, Y = np.meshgrid((p["start_iline"] + np.arange(kw["nx"])) * b, (p["start_xline"] + np.arange(kw["ny"])) * b,
                       indexing="ij")
    X, Y = X.ravel(), Y.ravel()
    t = np.arange(ns)
    v = synth.vrms_3d(X[:, None], (t * dt)[None, :], 1600.0, 500.0, 100.0, 8000.0)
    T = (ns - 1) * (1.0 + 2.0 ** -12)
    crit = (T * T - t[None, :] ** 2.0) * (v * dt) ** 2
    sx, sy, gx, gy = m.coords.T
    inap = ((X[None, :] - 0.5 * (sx + gx)[:, None]) ** 2 + (Y[None, :] - 0.5 * (sy + gy)[:, None]) ** 2
            < kw["aperture"] ** 2)
    D = (np.hypot(X[None, :] - sx[:, None], Y[None, :] - sy[:, None])
         + np.hypot(X[None, :] - gx[:, None], Y[None, :] - gy[:, None]))
    dead = sum((inap & (D * D >= crit[:, w0:w0 + window].max(1)[None, :])).sum() for w0 in range(0, ns, window))
    return dead / (inap.sum() * len(range(0, ns, window)))


@pytest.mark.parametrize("mode,K", [(capi.MODE_FULL, 8), (capi.MODE_FULL, 16), (capi.MODE_REFERENCE, 8),
                                    (capi.MODE_REFERENCE, 32)])
def test_dead_window_cull_is_invisible(kpstm_lib, mode, K):
    """The imaging kernel leaves out of a tile's trace list, per time
    window, the traces whose traveltimes lie past the trace end at every
    sample of the window, by sqrt(x + dS^2 y) + sqrt(x + dR^2 y) >=
    sqrt(4 x + (dS + dR)^2 y) with a 2^-12 margin.  Far offsets against
    short traces: over a tenth of the visits are dead; accumulators, fold
    counts and the pair count are identical with the cull turned off."""
    kw = dict(ntr=500, ns=401, dt=0.004, nx=12, ny=10, bin_m=25.0, max_offset=3500.0, n_refl=3, n_diff=10,
              freq=25.0, aperture=1500.0, aa_cutoff=60.0, seed=23, mode=mode, output=capi.OUT_STACK)
    assert _dead_window_share(synth.patch3d_model(**kw), kw, 32 * K) > 0.1
    s = synth.patch3d(**kw)
    out = []
    for cull in (1, 0):
        with Migration(s.params, s.velocity) as m:
            m.set_launch(samples_per_lane=K)
            assert kpstm_lib.kpstm_debug_trace_cull(m._h, cull) == 0
            m.add_traces(s.headers, s.samples)
            out.append((*m.accumulators(), m.pairs()))
    assert out[0][1].max() > 0
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32))
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
