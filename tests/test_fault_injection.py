"""Host-side fault injection (no GPU): malformed or truncated SEG-Y input
and a zero velocity reach the caller as status codes.  The reference exits
on these (Kirchhoff.c:462-467, 614-615) or ignores a short read
(:1280-1281); the ABI never exits."""
from __future__ import annotations

import ctypes as C
import tempfile
from pathlib import Path

import numpy as np

from random_gb300 import capi, synth
from random_gb300.migration import velocity_from_segy


def _files(s):
    td = Path(tempfile.mkdtemp())
    s.write_files(td / "d.segy", td / "v.segy")
    return (td / "d.segy").read_bytes(), (td / "v.segy").read_bytes()


def _info(lib, b):
    ns, dt, n = C.c_int32(), C.c_float(), C.c_int64()
    st = lib.kpstm_segy_info(b, len(b), C.byref(ns), C.byref(dt), C.byref(n))
    return st, ns.value, n.value


def test_truncated_data_file_counts_complete_traces(kpstm_lib):
    """A file cut inside a trace holds only its complete records, as
    count_size_file computes the trace count from the size (Kirchhoff.c:650-661)."""
    s = synth.line2d(n_cmp=6, n_off=4, ns=101, seed=2)
    data, _ = _files(s)
    rec = 240 + 4 * s.ns
    st, ns, n = _info(kpstm_lib, data)
    assert st == 0 and ns == s.ns and n == s.ntr
    st, _, n = _info(kpstm_lib, data[:-rec // 2])
    assert st == 0 and n == s.ntr - 1
    st, _, n = _info(kpstm_lib, data[:3600 + 3 * rec + 17])
    assert st == 0 and n == 3


def test_short_or_empty_header_is_a_segy_error(kpstm_lib):
    s = synth.line2d(n_cmp=4, n_off=2, ns=51, seed=2)
    data, _ = _files(s)
    assert _info(kpstm_lib, data[:3600 + 100])[0] == 10          # KPSTM_ERR_SEGY
    bad = bytearray(data)
    bad[3600 + 114:3600 + 118] = b"\x00\x00\x00\x00"             # ns = 0, dt = 0 in the first header
    assert _info(kpstm_lib, bytes(bad))[0] == 10


def test_truncated_velocity_file_reaches_the_zero_velocity_check(kpstm_lib):
    """The cut record of a truncated velocity file is never read, its grid
    cell stays 0, and kpstm_create refuses the model as the reference does
    (Kirchhoff.c:608-621) - before it looks for a device."""
    s = synth.line2d(n_cmp=6, n_off=4, ns=101, seed=2)
    _, vel = _files(s)
    v = s.velocity
    full, _, _ = velocity_from_segy(vel, v.n_iline, v.n_xline, v.o_iline, v.o_xline, v.d_iline, v.d_xline)
    assert np.array_equal(full, v.vrms.reshape(full.shape))
    rec = 240 + 4 * v.nsm
    cut, _, _ = velocity_from_segy(vel[:-rec // 3], v.n_iline, v.n_xline, v.o_iline, v.o_xline, v.d_iline,
                                   v.d_xline)
    assert np.all(cut.reshape(v.n_iline, -1)[-1] == 0) and np.array_equal(cut[:-1], full[:-1])
    vv = synth.Velocity(**{**v.__dict__, "vrms": cut.reshape(v.vrms.shape).astype(np.float32)})
    prm = capi.make_params(s.params)
    vel_s, _keep = capi.make_velocity(vv)
    h = C.c_void_p()
    assert kpstm_lib.kpstm_create(C.byref(prm), C.byref(vel_s), C.byref(h)) == 4  # KPSTM_ERR_VELOCITY_ZERO
    assert not h.value


def test_fail_alloc_hook_arguments(kpstm_lib):
    assert kpstm_lib.kpstm_debug_fail_alloc(-2) == 1
    assert kpstm_lib.kpstm_debug_fail_alloc(-1) == 0
    assert kpstm_lib.kpstm_debug_wait_limit(None, 0) == 1
