"""Error paths on the GPU without faulting it: a stage wait that gives up
(the test hook makes it give up at once, while the kernel still drains its
own copies with the full bound), device allocations that fail, and NaN
samples.  The reference exits on errors (Kirchhoff.c:462-467) and has no
device; here each error reaches the caller as a status and the context
stays usable."""
from __future__ import annotations

import numpy as np
import pytest

from random_gb300 import capi, synth
from random_gb300.migration import Migration, migrate

pytestmark = pytest.mark.gpu
TIMEOUT, OOM = 8, 3


def _line():
    return synth.line2d(n_cmp=24, n_off=8, ns=301, seed=9)


def _patch():
    return synth.patch3d(ntr=300, ns=201, dt=0.004, nx=8, ny=6, bin_m=25.0, max_offset=900.0, n_refl=2,
                         n_diff=4, freq=25.0, aperture=350.0, aa_cutoff=60.0, seed=13, mode=capi.MODE_FULL,
                         output=capi.OUT_STACK)


@pytest.mark.parametrize("make", [_line, _patch], ids=["reference-grid", "full-persistent"])
def test_stage_wait_timeout_is_reported_and_the_context_recovers(kpstm_lib, make):
    s = make()
    want = migrate(s, want_acc=True)
    with Migration(s.params, s.velocity) as m:
        assert kpstm_lib.kpstm_debug_wait_limit(m._h, 0) == 0
        m.add_traces(s.headers, s.samples)
        with pytest.raises(capi.KpstmError) as e:
            m.synchronize()
        assert e.value.status == TIMEOUT
        assert kpstm_lib.kpstm_debug_wait_limit(m._h, 1 << 22) == 0
        m.reset()
        m.add_traces(s.headers, s.samples)
        m.synchronize()
        km, fold = m.accumulators()
    assert np.array_equal(km.view(np.uint32), want["km"].view(np.uint32))
    assert np.array_equal(fold, want["fold"])


def test_failed_device_allocations_return_out_of_memory(kpstm_lib):
    """Every device allocation of the set-up and of the first block's
    staging, failed in turn: the call reports KPSTM_ERR_OUT_OF_MEMORY, and
    the job then runs to the same accumulators."""
    s = _line()
    want = migrate(s, want_acc=True)
    failed = 0
    try:
        for nth in range(64):
            assert kpstm_lib.kpstm_debug_fail_alloc(nth) == 0
            hit = False
            try:
                with Migration(s.params, s.velocity) as m:
                    try:
                        m.add_traces(s.headers, s.samples)
                    except capi.KpstmError as e:
                        assert e.status == OOM, e
                        hit = True
                        kpstm_lib.kpstm_debug_fail_alloc(-1)
                        m.add_traces(s.headers, s.samples)  # the same context, allocations working again
                    m.synchronize()
                    km, fold = m.accumulators()
                    assert np.array_equal(km.view(np.uint32), want["km"].view(np.uint32))
                    assert np.array_equal(fold, want["fold"])
            except capi.KpstmError as e:  # kpstm_create
                assert e.status == OOM, e
                hit = True
            kpstm_lib.kpstm_debug_fail_alloc(-1)
            failed += hit
            if not hit:
                break  # past the last allocation of the set-up and the first block
    finally:
        kpstm_lib.kpstm_debug_fail_alloc(-1)
    assert failed >= 10


def test_nan_samples_propagate_as_in_the_oracle(kpstm_lib, oracle_lib):
    """A NaN sample poisons that trace's running integrals from its sample
    on (Kirchhoff.c:1312-1328), in the reference as here: the accumulators
    are NaN exactly where the oracle's are and bit-equal elsewhere."""
    s = _line()
    s.samples = s.samples.copy()
    s.samples[37, 150] = np.nan
    g = migrate(s, want_acc=True)
    o = oracle_lib.kirchhoff(s)
    gn, on = np.isnan(g["km"]), np.isnan(o["km"])
    assert gn.any() and np.array_equal(gn, on)
    assert np.array_equal(g["km"][~gn].view(np.uint32), o["km"][~on].view(np.uint32))
    assert np.array_equal(g["fold"], o["fold"])
