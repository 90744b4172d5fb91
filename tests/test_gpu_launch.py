"""Launch configurations of the imaging kernel (kpstm_launch): tile patch
shape, samples per lane, persistent work queue, CUDA-graph replay of the
block pipeline, and the autotuner.

Every configuration changes only how the work is split; each image column
still sums its traces in block order, so the accumulators must be
bit-identical to the default launch.  The batched offset-class case (64
offset bins with Poisson trace counts, BF16 storage, one persistent launch
per block, graph replay, autotuned) is also checked against the FP64
oracle."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

from fixtures import rel_l2
from random_gb300 import capi, segy, synth
from random_gb300.migration import Migration

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _survey(mode, **kw):
    base = dict(ntr=600, ns=301, dt=0.004, nx=12, ny=10, bin_m=25.0, max_offset=1200.0, n_refl=3,
                n_diff=10, freq=25.0, aperture=450.0, aa_cutoff=60.0, seed=31, mode=mode,
                output=capi.OUT_OFFSET_GATHERS, nh=4, oh=0.0, dh=300.0)
    base.update(kw)
    return synth.patch3d(**base)


def _image(s, params=None, launch=None, block=250, device=False):
    p = dict(s.params)
    p.update(params or {})
    with Migration(p, s.velocity) as m:
        if launch:
            m.set_launch(**launch)
        hdr_be = np.ascontiguousarray(segy.headers_be(s.headers), dtype=np.int32)
        if device:
            dh = torch.from_numpy(hdr_be).cuda()
            ds = torch.from_numpy(np.ascontiguousarray(s.samples)).cuda()
            torch.cuda.synchronize()
        for b0 in range(0, s.ntr, block):
            b1 = min(s.ntr, b0 + block)
            if device:
                m.add_traces_device(dh[b0:b1].data_ptr(), ds[b0:b1].data_ptr(), b1 - b0)
            else:
                m.add_traces(s.headers[b0:b1], s.samples[b0:b1])
        km, fold = m.accumulators()
        return dict(km=km, fold=fold, pairs=m.pairs(), cfg=m.launch_config())


def _valid_K(mode, prec):
    kmax = 16 if prec == capi.PREC_BF16_KAHAN else (24 if mode == capi.MODE_FULL else 32)
    return [k for k in (8, 16, 24, 32) if k <= kmax]


@pytest.mark.parametrize("mode,prec", [(capi.MODE_REFERENCE, capi.PREC_FP32), (capi.MODE_FULL, capi.PREC_FP32),
                                       (capi.MODE_FULL, capi.PREC_BF16_KAHAN)])
def test_launch_configs_bit_identical(kpstm_lib, mode, prec):
    s = _survey(mode)
    prm = dict(precision=prec)
    ref = _image(s, prm)
    assert ref["pairs"] > 0
    full32 = mode == capi.MODE_FULL and prec == capi.PREC_FP32
    for px, K, pers, ctas in itertools.product((1, 2, 4, 8), _valid_K(mode, prec), (0, 1), (2, 3, 4)):
        if ctas == 3 and K > (16 if full32 else 8):
            continue
        if ctas == 4 and (not full32 or K > 8):
            continue
        g = _image(s, prm, dict(tile_px=px, samples_per_lane=K, persistent=pers, ctas_per_sm=ctas))
        assert g["cfg"]["tile_px"] == px and g["cfg"]["samples_per_lane"] == K
        assert g["cfg"]["ctas_per_sm"] == ctas
        assert np.array_equal(g["km"], ref["km"]), (px, K, pers, ctas)
        assert np.array_equal(g["fold"], ref["fold"]), (px, K, pers, ctas)
        assert g["pairs"] == ref["pairs"]


@pytest.mark.parametrize("device", [False, True])
def test_graph_replay_bit_identical(kpstm_lib, device):
    """Blocks of 250, 250, 100 traces: the two staging slots and the short
    last block each capture a graph; replays must equal direct launches."""
    s = _survey(capi.MODE_FULL)
    ref = _image(s, device=device)
    for pers in (0, 1):
        g = _image(s, launch=dict(graph=1, persistent=pers), device=device)
        assert g["cfg"]["graph"] == 1
        assert np.array_equal(g["km"], ref["km"]) and np.array_equal(g["fold"], ref["fold"])


def test_graph_replay_on_a_caller_stream(kpstm_lib):
    """Graph capture and replay on the caller's stream (kpstm_set_stream):
    the same accumulators as direct launches on the context's own stream."""
    s = _survey(capi.MODE_FULL)
    ref = _image(s, device=True)
    hdr_be = np.ascontiguousarray(segy.headers_be(s.headers), dtype=np.int32)
    dh = torch.from_numpy(hdr_be).cuda()
    ds = torch.from_numpy(np.ascontiguousarray(s.samples)).cuda()
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    with Migration(s.params, s.velocity) as m:
        m.set_stream(stream.cuda_stream)
        m.set_launch(graph=1)
        for b0 in range(0, s.ntr, 250):
            b1 = min(s.ntr, b0 + 250)
            m.add_traces_device(dh[b0:b1].data_ptr(), ds[b0:b1].data_ptr(), b1 - b0)
        km, fold = m.accumulators()
    assert np.array_equal(km, ref["km"]) and np.array_equal(fold, ref["fold"])


def test_set_launch_rejects_bad_values(kpstm_lib):
    s = _survey(capi.MODE_FULL, ntr=10)
    with Migration(s.params, s.velocity) as m:
        for bad in (dict(tile_px=3), dict(samples_per_lane=32), dict(samples_per_lane=12), dict(persistent=2),
                    dict(graph=-1), dict(ctas_per_sm=5), dict(ctas_per_sm=3, samples_per_lane=24),
                    dict(ctas_per_sm=4, samples_per_lane=16)):
            with pytest.raises(capi.KpstmError) as e:
                m.set_launch(**bad)
            assert e.value.status == 1  # KPSTM_ERR_INVALID_ARG


def test_autotune(kpstm_lib):
    s = _survey(capi.MODE_FULL)
    ref = _image(s)
    hdr_be = np.ascontiguousarray(segy.headers_be(s.headers), dtype=np.int32)
    dh = torch.from_numpy(hdr_be).cuda()
    ds = torch.from_numpy(np.ascontiguousarray(s.samples)).cuda()
    torch.cuda.synchronize()
    with Migration(s.params, s.velocity) as m:
        m.set_launch(graph=1)
        cfg, ms = m.autotune(dh.data_ptr(), ds.data_ptr(), 200)
        assert ms > 0.0
        assert cfg["tile_px"] in (1, 2, 4, 8) and cfg["samples_per_lane"] in (8, 16, 24)
        assert cfg["graph"] == 1 and m.launch_config() == cfg
        km, fold = m.accumulators()
        assert not km.any() and np.all(fold == 1.0) and m.pairs() == 0  # cleared again
        for b0 in range(0, s.ntr, 250):
            b1 = min(s.ntr, b0 + 250)
            m.add_traces_device(dh[b0:b1].data_ptr(), ds[b0:b1].data_ptr(), b1 - b0)
        km, fold = m.accumulators()
        assert np.array_equal(km, ref["km"]) and np.array_equal(fold, ref["fold"])
        with pytest.raises(capi.KpstmError) as e:  # traces imaged since create
            m.autotune(dh.data_ptr(), ds.data_ptr(), 200)
        assert e.value.status == 7  # KPSTM_ERR_STATE


def test_batched_offset_bins(kpstm_lib, oracle_lib):
    """64 offset bins over 0-4000 m with Poisson trace counts, BF16 storage
    with Kahan accumulation, persistent launch + graph, autotuned; reduced
    sizes (Poisson(40) per bin, 16 x 16 image, 1001 samples at 4 ms)."""
    counts = synth.offset_bin_counts(64, 40.0, 10, 100, seed=7)
    mdl = synth.offset_bins_model(counts, nx=16, ny=16, bin_m=12.5, aperture=150.0, n_refl=3, n_diff=20,
                                  mode=capi.MODE_REFERENCE, aa_cutoff=1e6)
    s = mdl.survey
    s.samples = synth.synthesize_numpy(mdl)
    prm = dict(precision=capi.PREC_BF16_KAHAN)
    base = _image(s, prm, block=1000)
    hdr_be = np.ascontiguousarray(segy.headers_be(s.headers), dtype=np.int32)
    dh = torch.from_numpy(hdr_be).cuda()
    ds = torch.from_numpy(np.ascontiguousarray(s.samples)).cuda()
    torch.cuda.synchronize()
    p = dict(s.params)
    p.update(prm)
    with Migration(p, s.velocity) as m:
        m.set_launch(persistent=1, graph=1)
        m.autotune(dh.data_ptr(), ds.data_ptr(), 500)
        m.set_launch(**dict(m.launch_config(), persistent=1, graph=1))
        for b0 in range(0, s.ntr, 1000):
            b1 = min(s.ntr, b0 + 1000)
            m.add_traces_device(dh[b0:b1].data_ptr(), ds[b0:b1].data_ptr(), b1 - b0)
        km, fold = m.accumulators()
        pairs = m.pairs()
    assert np.array_equal(km, base["km"]) and np.array_equal(fold, base["fold"])
    assert pairs == base["pairs"] > 0
    # every bin received its traces: fold > 1 somewhere in each class
    assert np.all(fold.reshape(16 * 16, 64, -1).max(axis=(0, 2)) > 1.0)
    o = oracle_lib.kirchhoff64(s)
    assert rel_l2(km, o["km"]) <= 2e-2, rel_l2(km, o["km"])
