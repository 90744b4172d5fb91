"""The headline workload at its full image size (400 x 400 x 1501 stack at
25 m, 1501 samples at 2 ms, 3000 m aperture, full physics), checked through
properties that hold at any size, on a 10,000-trace block of the same
survey (the FP64 oracle cannot run at this size):

* linearity in the data: L^T(a d1 + d2) = a L^T d1 + L^T d2 for two
  band-limited datasets (the events of two seeded surveys on the same
  geometry), up to the rounding of the fp32 tap tables and sums (bar 5e-5
  relative L2; white noise would not do: its double running integral grows
  like n^1.5 and the fp32 table of it loses ~1e-3 of the taps);
* the pair count equals an independent count of the in-aperture
  (trace, column) pairs with the float32 test of Kirchhoff.c:1351-1354;
* a block split is invisible: two 5,000-trace blocks give the same
  accumulators as one 10,000-trace block, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from fixtures import rel_l2
from random_gb300 import capi, segy, synth
from random_gb300.migration import Migration

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

NTR = 10_000


def _model(seed):
    return synth.patch3d_model(1_000_000, ns=1501, dt=0.002, nx=400, ny=400, bin_m=25.0, max_offset=4000.0,
                               n_refl=8, n_diff=200, freq=30.0, aperture=3000.0, aa_cutoff=100.0, seed=seed,
                               mode=capi.MODE_FULL, output=capi.OUT_STACK, trace_slice=slice(0, NTR))


@pytest.fixture(scope="module")
def survey():
    m = _model(2)
    d = synth.synthesize_torch(m, device="cuda")
    hdr = torch.from_numpy(np.ascontiguousarray(segy.headers_be(m.survey.headers), dtype=np.int32)).cuda()
    torch.cuda.synchronize()
    return m.survey, hdr, d


def _accumulate(s, hdr, d, blocks):
    with Migration(s.params, s.velocity) as m:
        b0 = 0
        for n in blocks:
            m.add_traces_device(hdr[b0:b0 + n].data_ptr(), d[b0:b0 + n].data_ptr(), n)
            b0 += n
        km, fold = m.accumulators()
        return km, fold, m.pairs()


def test_linearity_in_the_data(kpstm_lib, survey):
    s, hdr, d1 = survey
    m2 = _model(7)  # other events; the same geometry (the trace draws come first)
    m2.coords = _model(2).coords
    d2 = synth.synthesize_torch(m2, device="cuda")
    a = 0.75
    k1, f1, p1 = _accumulate(s, hdr, d1.contiguous(), [NTR])
    k2, f2, _ = _accumulate(s, hdr, d2.contiguous(), [NTR])
    k3, f3, _ = _accumulate(s, hdr, (a * d1 + d2).contiguous(), [NTR])
    assert p1 > 0 and np.array_equal(f1, f2) and np.array_equal(f1, f3)
    assert rel_l2(k3, a * k1.astype(np.float64) + k2) <= 5e-5


def test_pair_count_is_exact(kpstm_lib, survey):
    s, hdr, d = survey
    _, _, pairs = _accumulate(s, hdr, d, [NTR])
    p = s.params
    h = s.headers.astype(np.float64)
    cx = (0.5 * (h[:, 18] + h[:, 20])).astype(np.float32)
    cy = (0.5 * (h[:, 19] + h[:, 21])).astype(np.float32)
    IX = ((p["start_iline"] + np.arange(400)) * 25.0).astype(np.float32)
    IY = ((p["start_xline"] + np.arange(400)) * 25.0).astype(np.float32)
    n = 0
    for i in range(0, NTR, 500):
        dx = IX[None, :] - cx[i:i + 500, None]                      # [tr, x]
        dy = IY[None, :] - cy[i:i + 500, None]                      # [tr, y]
        d2 = dx[:, :, None] * dx[:, :, None] + dy[:, None, :] * dy[:, None, :]
        n += int((np.sqrt(d2) < np.float32(3000.0)).sum())
    assert pairs == n * 1501


def test_block_split_is_invisible(kpstm_lib, survey):
    s, hdr, d = survey
    k1, f1, p1 = _accumulate(s, hdr, d, [NTR])
    k2, f2, p2 = _accumulate(s, hdr, d, [NTR // 2, NTR // 2])
    assert p1 == p2 and np.array_equal(k1, k2) and np.array_equal(f1, f2)
