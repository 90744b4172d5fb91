"""The imaging kernel's dead-window trace cull, checked on the CPU: the
kernel leaves a trace out of an image tile's list for a time window when
its summed source and receiver distances to the tile's box of column
positions satisfy D^2 >= crit, crit the largest over the tile's columns and
the window's samples of (T^2 - 4 x) / y (full mode, sample units) or
(T^2 - 4 t2) v2 (reference mode, seconds), with T a 2^-12 margin past the
last sample.  This test evaluates the bound in float32 as the kernel does
and then the kernel's own traveltime arithmetic for every column and sample
of each culled (trace, tile, window) - with every SFU reciprocal square root
taken at its worst-case error, 2^-21 low - and asserts that none of those
pairs would have been imaged.  The GPU test that the images do not change
with the cull turned off is test_gpu_full_mode.test_dead_window_cull_is_invisible."""
from __future__ import annotations

import numpy as np
import pytest

f32, f64 = np.float32, np.float64
MARGIN = f32(1.0 + 1.0 / 4096.0)
RSQ_LOW = f32(1.0 - 2.0 ** -21)


def _fma(a, b, c):
    """fp32 fma: the exact product of two floats fits a double."""
    return (f64(a) * f64(b) + f64(c)).astype(f32)


def _geometry(rng, ntile, ntr, spread):
    """Tiles of 4 x 2 columns at 25 m (float32 positions, as the column
    table holds them) and traces with source and receiver anywhere within
    `spread` metres of the tile."""
    ox = rng.uniform(1e4, 2e4, ntile)
    oy = rng.uniform(1e4, 2e4, ntile)
    cx = (ox[:, None] + 25.0 * np.repeat(np.arange(4), 2)[None, :]).astype(f32)   # [tile, 8]
    cy = (oy[:, None] + 25.0 * np.tile(np.arange(2), 4)[None, :]).astype(f32)
    box = np.stack([cx.min(1), cx.max(1), cy.min(1), cy.max(1)], 1)              # xmin, xmax, ymin, ymax
    s = (np.stack([ox, oy], 1)[:, None, None, :] +
         rng.uniform(-spread, spread, (ntile, ntr, 2, 2))).astype(f32)            # [tile, tr, S|R, xy]
    return cx, cy, box, s


def _box_dist(box, x, y):
    dx = np.maximum(np.maximum(box[:, None, 0] - x, x - box[:, None, 1]), f32(0))
    dy = np.maximum(np.maximum(box[:, None, 2] - y, y - box[:, None, 3]), f32(0))
    return np.sqrt(dx * dx + dy * dy)


def _distances(cx, cy, s):
    """The kernel's squared source and receiver distances per (tile, trace, column)."""
    sx = cx[:, None, :] - s[:, :, 0, 0][:, :, None]
    sy = cy[:, None, :] - s[:, :, 0, 1][:, :, None]
    gx = cx[:, None, :] - s[:, :, 1, 0][:, :, None]
    gy = cy[:, None, :] - s[:, :, 1, 1][:, :, None]
    return sx * sx + sy * sy, gx * gx + gy * gy


@pytest.mark.parametrize("ns,dt,window", [(401, 0.004, 256), (401, 0.004, 512), (751, 0.004, 512),
                                          (1501, 0.002, 512)])
def test_full_mode_cull_leaves_out_only_dead_pairs(ns, dt, window):
    rng = np.random.default_rng(ns + window)
    ntile, ntr = 24, 160
    cx, cy, box, s = _geometry(rng, ntile, ntr, 6000.0)
    t = np.arange(ns)
    tx = np.where(t > 0, (0.25 * t.astype(f64) ** 2), 1e-12).astype(f32)
    rdt = f32(f32(1.0) / f32(dt))
    rdt2 = f32(rdt * rdt)
    v = (1500.0 + 900.0 * t * dt)[None, None, :] + 80.0 * np.sin(cx.astype(f64) / 700.0)[:, :, None]
    vv = (v * v).astype(f32)                                                      # [tile, col, t]
    ty = f32(1.0) / vv * rdt2
    tmax = f32(ns - 1)
    T = f32(tmax * MARGIN)
    crit_t = (f32(T * T) - f32(4.0) * tx[None, None, :]) / ty                     # [tile, col, t]
    D = _box_dist(box, s[:, :, 0, 0], s[:, :, 0, 1]) + _box_dist(box, s[:, :, 1, 0], s[:, :, 1, 1])
    dS2, dR2 = _distances(cx, cy, s)
    culled = 0
    for w0 in range(0, ns, window):
        w1 = min(ns, w0 + window)
        crit = crit_t[:, :, w0:w1].max(axis=(1, 2))                               # [tile]
        cull = (D * D) >= crit[:, None]                                           # [tile, tr]
        ti, tr = np.nonzero(cull)
        culled += len(ti)
        if not len(ti):
            continue
        a_s = _fma(dS2[ti, tr][:, :, None], ty[ti][:, :, w0:w1], tx[None, None, w0:w1])
        a_r = _fma(dR2[ti, tr][:, :, None], ty[ti][:, :, w0:w1], tx[None, None, w0:w1])
        rs = (f32(1.0) / np.sqrt(a_s)) * RSQ_LOW
        rr = (f32(1.0) / np.sqrt(a_r)) * RSQ_LOW
        tf = _fma(a_s, rs, a_r * rr)
        assert np.all(tf >= tmax), float(tf.min())
    assert culled > 0.05 * ntile * ntr * len(range(0, ns, window))


@pytest.mark.parametrize("ns,dt,window", [(401, 0.004, 256), (1001, 0.004, 768)])
def test_reference_mode_cull_leaves_out_only_dead_pairs(ns, dt, window):
    rng = np.random.default_rng(7 * ns + window)
    ntile, ntr = 24, 160
    cx, cy, box, s = _geometry(rng, ntile, ntr, 6000.0)
    t = np.arange(ns)
    dtf = f32(dt)
    t2 = (0.25 * t.astype(f64) ** 2 * f64(dtf) ** 2).astype(f32)
    v = (1500.0 + 900.0 * t * dt)[None, None, :] + 80.0 * np.sin(cx.astype(f64) / 700.0)[:, :, None]
    v2 = (v * v).astype(f32)
    nsf = f32(ns)
    T = f32(f32(nsf * dtf) * MARGIN)
    crit_t = (f32(T * T) - f32(4.0) * t2[None, None, :]) * v2
    D = _box_dist(box, s[:, :, 0, 0], s[:, :, 0, 1]) + _box_dist(box, s[:, :, 1, 0], s[:, :, 1, 1])
    dS2, dR2 = _distances(cx, cy, s)
    culled = 0
    for w0 in range(0, ns, window):
        w1 = min(ns, w0 + window)
        crit = crit_t[:, :, w0:w1].max(axis=(1, 2))
        cull = (D * D) >= crit[:, None]
        ti, tr = np.nonzero(cull)
        culled += len(ti)
        if not len(ti):
            continue
        # RN(d / v2), RN(t2 + q), the double square roots summed in double and
        # rounded to float (Kirchhoff.c:1383), then RN(S / dt) against ns
        q1 = dS2[ti, tr][:, :, None] / v2[ti][:, :, w0:w1]
        q2 = dR2[ti, tr][:, :, None] / v2[ti][:, :, w0:w1]
        a1 = t2[None, None, w0:w1] + q1
        a2 = t2[None, None, w0:w1] + q2
        S = (np.sqrt(a1.astype(f64)) + np.sqrt(a2.astype(f64))).astype(f32)
        assert np.all(S / dtf >= nsf), float((S / dtf).min())
    assert culled > 0.05 * ntile * ntr * len(range(0, ns, window))
