"""Least-squares migration: the GPU operator pair (migration L^T, its
transpose L, demigration) against the FP64 oracle operators, the adjoint
dot-product test, finite-difference checks of the misfit gradient, and CG
against an FP64 CGLS driven by the oracle operators.  No reference
counterpart: the reference migrates once and has no adjoint."""
from __future__ import annotations

import numpy as np
import pytest

from fixtures import rel_l2
from random_gb300 import capi, synth
from random_gb300.migration import Migration

pytestmark = pytest.mark.gpu


def _survey(**kw):
    base = dict(ntr=240, ns=201, dt=0.004, nx=8, ny=6, bin_m=25.0, max_offset=900.0, n_refl=2, n_diff=6,
                freq=25.0, aperture=350.0, aa_cutoff=60.0, seed=31, mode=capi.MODE_FULL, output=capi.OUT_STACK)
    base.update(kw)
    return synth.patch3d(**base)


class Ops:
    """GPU operator pair on torch device vectors."""

    def __init__(self, s, **p):
        import torch
        self.t = torch
        self.m = Migration(dict(s.params, **p), s.velocity)
        self.m.lsm_geometry(s.headers)
        self.dshape = (s.ntr, s.ns)
        self.mshape = self.m.shape

    def adj(self, d):
        d = self.t.as_tensor(np.ascontiguousarray(d, np.float32)).cuda()
        out = self.t.empty(self.mshape, dtype=self.t.float32, device="cuda")
        self.t.cuda.synchronize()
        self.m.lsm_adjoint(d.data_ptr(), out.data_ptr())
        return out.cpu().numpy().astype(np.float64)

    def fwd(self, m):
        m = self.t.as_tensor(np.ascontiguousarray(m, np.float32)).cuda()
        out = self.t.empty(self.dshape, dtype=self.t.float32, device="cuda")
        self.t.cuda.synchronize()
        self.m.lsm_forward(m.data_ptr(), out.data_ptr())
        return out.cpu().numpy().astype(np.float64)


@pytest.fixture(scope="module")
def setup(kpstm_lib):
    pytest.importorskip("torch")
    s = _survey()
    return s, Ops(s)


def test_operators_match_fp64_oracle(setup, oracle_lib):
    s, ops = setup
    rng = np.random.default_rng(1)
    d = rng.normal(size=ops.dshape)
    m = rng.normal(size=ops.mshape)
    assert rel_l2(ops.adj(d), oracle_lib.lsm_apply(s, 0, d)) <= 1e-4
    assert rel_l2(ops.fwd(m), oracle_lib.lsm_apply(s, 1, m)) <= 1e-4


def test_dot_product(setup):
    s, ops = setup
    rng = np.random.default_rng(2)
    for _ in range(3):
        d = rng.normal(size=ops.dshape)
        m = rng.normal(size=ops.mshape)
        a = np.vdot(ops.adj(d), m)
        b = np.vdot(d, ops.fwd(m))
        assert abs(a - b) <= 1e-5 * max(abs(a), abs(b)), (a, b)


def test_misfit_gradient_finite_differences(setup):
    """J(m) = |L m - d|^2 / 2, grad = L^T (L m - d): central differences along
    16 random directions (J is quadratic, so the central difference is exact
    up to rounding)."""
    s, ops = setup
    rng = np.random.default_rng(3)
    d = ops.fwd(rng.normal(size=ops.mshape)) + 0.1 * rng.normal(size=ops.dshape)
    m = rng.normal(size=ops.mshape)
    J = lambda mm: 0.5 * float(np.sum((ops.fwd(mm) - d) ** 2))
    g = ops.adj(ops.fwd(m) - d)
    for _ in range(16):
        dm = rng.normal(size=ops.mshape)
        h = 1e-2 * np.linalg.norm(m) / np.linalg.norm(dm)
        fd = (J(m + h * dm) - J(m - h * dm)) / (2 * h)
        an = float(np.vdot(g, dm))
        assert abs(fd - an) <= 2e-3 * abs(an) + 1e-9 * np.linalg.norm(g) * np.linalg.norm(dm), (fd, an)


def _cgls(apply_L, apply_LT, d, niter):
    x = np.zeros_like(apply_LT(np.zeros_like(d)))
    r = d.copy()
    s_ = apply_LT(r)
    p = s_.copy()
    gamma = np.vdot(s_, s_)
    res = [np.linalg.norm(r)]
    for _ in range(niter):
        q = apply_L(p)
        alpha = gamma / np.vdot(q, q)
        x += alpha * p
        r -= alpha * q
        res.append(np.linalg.norm(r))
        s_ = apply_LT(r)
        gnew = np.vdot(s_, s_)
        p = s_ + (gnew / gamma) * p
        gamma = gnew
    return x, np.array(res)


@pytest.mark.parametrize("precision", [capi.PREC_FP32, capi.PREC_BF16_KAHAN])
def test_cg_against_fp64_oracle(kpstm_lib, oracle_lib, precision):
    torch = pytest.importorskip("torch")
    s = _survey(ntr=180, nx=6, ny=5)
    rng = np.random.default_rng(4)
    m_true = np.zeros((6, 5, 1, s.ns))
    m_true[:, :, 0, 60] = 1.0
    m_true[2, 3, 0, 120] = -2.0
    d = oracle_lib.lsm_apply(s, 1, m_true)
    d += 0.05 * np.std(d) * rng.normal(size=d.shape)
    niter = 8
    x64, res64 = _cgls(lambda v: oracle_lib.lsm_apply(s, 1, v), lambda v: oracle_lib.lsm_apply(s, 0, v), d, niter)
    with Migration(dict(s.params, precision=precision), s.velocity) as mg:
        mg.lsm_geometry(s.headers)
        dd = torch.as_tensor(d.astype(np.float32)).cuda()
        xm = torch.empty(mg.shape, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        res = mg.lsm_cg(dd.data_ptr(), niter, xm.data_ptr())
        x = xm.cpu().numpy()
    assert np.all(np.diff(res) <= 1e-6 * res[0])          # residual never grows
    err = rel_l2(x, x64)
    assert err <= (1e-3 if precision == capi.PREC_FP32 else 2e-2), err


def test_cg_monitor_iterates_and_stop(kpstm_lib):
    """kpstm_lsm_cg_ex: the iterate the monitor sees after iteration k equals
    a separate k-iteration solve bit for bit (CGLS from m = 0 is the same
    recurrence), residuals agree, and a truthy return ends the solve."""
    torch = pytest.importorskip("torch")
    s = _survey(ntr=180, nx=6, ny=5)
    rng = np.random.default_rng(5)
    d = torch.as_tensor(rng.normal(size=(s.ntr, s.ns)).astype(np.float32)).cuda()
    with Migration(dict(s.params, precision=capi.PREC_BF16_KAHAN), s.velocity) as mg:
        mg.lsm_geometry(s.headers)
        xm = torch.empty(mg.shape, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        seen, res_seen = [], []

        def mon(k, ptr, res):
            assert ptr == xm.data_ptr()
            seen.append(xm.cpu().numpy().copy())
            res_seen.append(res)
            return False
        resid = mg.lsm_cg(d.data_ptr(), 4, xm.data_ptr(), monitor=mon)
        assert len(seen) == 4 and len(resid) == 5
        assert np.allclose(res_seen, resid[1:], rtol=0, atol=0)
        for k in (1, 3):
            r2 = mg.lsm_cg(d.data_ptr(), k, xm.data_ptr())
            assert np.array_equal(xm.cpu().numpy(), seen[k - 1])
            assert np.array_equal(r2, resid[:k + 1])
        stop = []
        r3 = mg.lsm_cg(d.data_ptr(), 6, xm.data_ptr(), monitor=lambda k, p, r: stop.append(k) or k == 2)
        assert stop == [1, 2] and len(r3) == 3
        assert np.array_equal(xm.cpu().numpy(), seen[1])
        r0 = mg.lsm_cg(d.data_ptr(), 0, xm.data_ptr())
        assert len(r0) == 1 and not np.any(xm.cpu().numpy())
