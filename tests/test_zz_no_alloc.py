"""kpstm_finish_noalloc: the finishing step for callers that must not
allocate device memory (their framework's allocator already owns the memory
they may use, or cudaMalloc/cudaFree would synchronise a pipelined device).

Checked through the C ABI against the regular kpstm_finish, on two calls in
a row (the second call reuses the library's fixed scratch array left over
from the first).  This file is collected last on purpose; every test in it
builds what it needs, so it also passes alone in a fresh process."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from fixtures import load, rel_l2
from random_gb300 import capi
from random_gb300.migration import Migration

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _accumulators(name="g1_line_oddns", **over):
    s, *_ = load(name)
    p = dict(s.params, **over)
    with Migration(p, s.velocity) as m:
        m.add_traces(s.headers, s.samples)
        km, fold = m.accumulators()
        image = m.finish()
    return p, km, fold, image


def test_noalloc_finish_matches_kpstm_finish_twice(kpstm_lib):
    torch = pytest.importorskip("torch")
    p, km, fold, image = _accumulators()
    d_km = torch.from_numpy(km).cuda()
    d_fold = torch.from_numpy(fold).cuda()
    prm = capi.make_params(p)
    outs = []
    for _ in range(2):
        d_out = torch.full(km.shape, float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        st = kpstm_lib.kpstm_finish_noalloc(C.byref(prm), d_km.data_ptr(), d_fold.data_ptr(),
                                            d_out.data_ptr(), None)
        assert st == 0, capi.STATUS.get(st, st)
        torch.cuda.synchronize()
        outs.append(d_out.cpu().numpy())
    for out in outs:
        assert np.all(np.isfinite(out))
        assert rel_l2(out, image) <= TOL
    assert np.array_equal(outs[0], outs[1])


def test_noalloc_finish_even_ns_low_pass(kpstm_lib):
    """Even ns and a real anti-alias cutoff, after a different-size call."""
    torch = pytest.importorskip("torch")
    p, km, fold, image = _accumulators("g2_line_slabs")
    d_km, d_fold = torch.from_numpy(km).cuda(), torch.from_numpy(fold).cuda()
    d_out = torch.empty_like(d_km)
    prm = capi.make_params(p)
    torch.cuda.synchronize()
    assert kpstm_lib.kpstm_finish_noalloc(C.byref(prm), d_km.data_ptr(), d_fold.data_ptr(),
                                          d_out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert rel_l2(d_out.cpu().numpy(), image) <= TOL


def test_noalloc_finish_refuses_images_beyond_its_scratch(kpstm_lib):
    torch = pytest.importorskip("torch")
    s, *_ = load("g1_line_oddns")
    # 2100 x 1 x 8 x 251 samples > KPSTM_NOALLOC_MAX_SAMPLES
    p = dict(s.params, end_iline=s.params["start_iline"] + 2100, nh=8)
    n = 2100 * 8 * s.ns
    assert n > capi.NOALLOC_MAX_SAMPLES
    d = torch.zeros(8, dtype=torch.float32, device="cuda")  # never touched
    prm = capi.make_params(p)
    st = kpstm_lib.kpstm_finish_noalloc(C.byref(prm), d.data_ptr(), d.data_ptr(), d.data_ptr(), None)
    assert st == 13  # KPSTM_ERR_TOO_LARGE
    assert b"noalloc" in kpstm_lib.kpstm_strerror(13)


def test_noalloc_finish_full_mode_offset_classes(kpstm_lib):
    """Full physics on the rotated 3-D patch with 4 offset classes: the
    accumulators arrive scaled by t/(8 dt) per sample, as
    kpstm_get_accumulators returns them, and finish like kpstm_finish."""
    torch = pytest.importorskip("torch")
    p, km, fold, image = _accumulators("g3_patch_rotated", mode=capi.MODE_FULL)
    assert km.shape[2] == 4
    d_km, d_fold = torch.from_numpy(km).cuda(), torch.from_numpy(fold).cuda()
    prm = capi.make_params(p)
    for _ in range(2):
        d_out = torch.full(km.shape, float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        assert kpstm_lib.kpstm_finish_noalloc(C.byref(prm), d_km.data_ptr(), d_fold.data_ptr(),
                                              d_out.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert rel_l2(d_out.cpu().numpy(), image) <= TOL


def test_noalloc_finish_refuses_long_traces(kpstm_lib):
    """ns beyond KPSTM_NOALLOC_MAX_NS (the low-pass kernel's shared memory) is
    refused even for a one-column image."""
    torch = pytest.importorskip("torch")
    s, *_ = load("g1_line_oddns")
    p = dict(s.params, ns=capi.NOALLOC_MAX_NS + 1, end_iline=s.params["start_iline"] + 1, nh=1)
    d = torch.zeros(8, dtype=torch.float32, device="cuda")  # never touched
    prm = capi.make_params(p)
    st = kpstm_lib.kpstm_finish_noalloc(C.byref(prm), d.data_ptr(), d.data_ptr(), d.data_ptr(), None)
    assert st == 13  # KPSTM_ERR_TOO_LARGE
