"""C-ABI checks that need no GPU: the library builds and loads, exports every
function include/kpstm.h declares, and its host-only helpers agree with the
oracle / the reference formulas."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from fixtures import load
from random_gb300 import capi, segy, synth

HEADER = Path(__file__).resolve().parents[1] / "include" / "kpstm.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(kpstm_\w+)\s*\(", text)))


def test_header_declares_the_abi():
    names = declared_functions()
    for must in ["kpstm_create", "kpstm_add_traces", "kpstm_add_segy_block", "kpstm_add_traces_device",
                 "kpstm_finish", "kpstm_destroy", "kpstm_strerror"]:
        assert must in names


def test_library_exports_every_declared_symbol(kpstm_lib):
    missing = [n for n in declared_functions() if not hasattr(kpstm_lib, n)]
    assert not missing, missing


def test_abi_version_and_strerror(kpstm_lib):
    assert kpstm_lib.kpstm_abi_version() == 1
    for code in range(14):
        assert kpstm_lib.kpstm_strerror(code)


def test_struct_sizes_match_header_layout():
    # natural alignment of the C structs in include/kpstm.h
    assert C.sizeof(capi.KpstmParams) == 184
    assert C.sizeof(capi.KpstmDims) == 48


def test_ctypes_layouts_match_the_c_compiler(tmp_path):
    """Every ABI struct: sizeof and each field offset as gcc lays them out
    from include/kpstm.h, against the ctypes mirror."""
    structs = {"kpstm_params": capi.KpstmParams, "kpstm_velocity": capi.KpstmVelocity,
               "kpstm_dims": capi.KpstmDims, "kpstm_profile": capi.KpstmProfile, "kpstm_launch": capi.KpstmLaunch}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "kpstm.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{HEADER.parent}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    for line in filter(None, out):
        cname, what, val = line.split()
        py = structs[cname]
        want = C.sizeof(py) if what == "sizeof" else getattr(py, what).offset
        assert int(val) == want, line


def test_aliasfilter_matches_oracle(kpstm_lib, oracle_lib):
    for ns, dt, a, b, cut in [(1001, 0.004, 25.0, 25.0, 1e6), (1501, 0.002, 25.0, 12.5, 50.0),
                              (300, 0.004, 12.5, 25.0, 40.0), (751, 0.004, 50.0, 50.0, 10.0)]:
        aa = np.zeros(ns, np.float32)
        tm = C.c_int32()
        capi.check("aliasfilter", kpstm_lib.kpstm_aliasfilter(ns, np.float32(dt), a, b, cut, C.byref(tm),
                                                              aa.ctypes.data))
        tmo, aao = oracle_lib.aliasfilter(ns, np.float32(dt), a, b, cut)
        assert tm.value == tmo
        assert np.array_equal(aa, aao)


def test_ibm_decode_matches_reference_formula(kpstm_lib):
    rng = np.random.default_rng(3)
    x = (rng.normal(size=5000) * 10.0 ** rng.uniform(-30, 30, 5000)).astype(np.float32)
    x[:4] = [0.0, -0.0, 1.0, -1.0]
    words = segy.ieee_to_ibm(x)
    be = words.astype(">u4").view(np.uint32)
    out = np.zeros(x.size, np.float32)
    capi.check("ibm", kpstm_lib.kpstm_ibm_to_ieee(be.ctypes.data, out.ctypes.data, x.size))
    assert np.array_equal(out.view(np.uint32), segy.ibm_to_ieee(words).view(np.uint32))
    # tiny exponents: 16^(e-64) underflows to subnormal / zero as in float
    w = np.array([0x00100000 | (e << 24) for e in range(0, 40)], np.uint32)
    out = np.zeros(w.size, np.float32)
    kpstm_lib.kpstm_ibm_to_ieee(w.astype(">u4").view(np.uint32).ctypes.data, out.ctypes.data, w.size)
    assert np.array_equal(out, segy.ibm_to_ieee(w))


def test_segy_info(kpstm_lib, tmp_path):
    s = synth.line2d(n_cmp=4, n_off=3, ns=77, seed=1)
    s.write_files(tmp_path / "d.segy", tmp_path / "v.segy")
    raw = np.fromfile(tmp_path / "d.segy", np.uint8)
    ns, dt, ntr = C.c_int32(), C.c_float(), C.c_int64()
    capi.check("info", kpstm_lib.kpstm_segy_info(raw.ctypes.data, raw.size, C.byref(ns), C.byref(dt), C.byref(ntr)))
    assert (ns.value, ntr.value) == (77, 12)
    assert dt.value == np.float32(0.004)
    assert kpstm_lib.kpstm_segy_info(raw.ctypes.data, 100, None, None, None) == 10


def test_create_rejects_bad_arguments_without_touching_a_gpu(kpstm_lib):
    s, *_ = load("g1_line_oddns")
    bad = dict(s.params, ns=0)
    prm = capi.make_params(bad)
    vel, keep = capi.make_velocity(s.velocity)
    h = C.c_void_p()
    assert kpstm_lib.kpstm_create(C.byref(prm), C.byref(vel), C.byref(h)) == 1
    # trangeMax < 2 (fine line spacing) is refused, as the taps would leave the trace
    prm = capi.make_params(dict(s.params, iline_distance=0.5, xline_distance=0.5))
    assert kpstm_lib.kpstm_create(C.byref(prm), C.byref(vel), C.byref(h)) == 12
    # zero velocity sample (Kirchhoff.c:614-615)
    v0 = s.velocity.vrms.copy()
    v0[0, 0, 5] = 0.0
    vel0 = capi.KpstmVelocity(s.velocity.n_iline, s.velocity.n_xline, s.velocity.nsm, s.velocity.o_iline,
                              s.velocity.o_xline, s.velocity.d_iline, s.velocity.d_xline, s.velocity.dtm,
                              v0.ctypes.data)
    prm = capi.make_params(s.params)
    assert kpstm_lib.kpstm_create(C.byref(prm), C.byref(vel0), C.byref(h)) == 4
    # velocity interpolation exists for the full operator only (reference mode is exact)
    prm = capi.make_params(dict(s.params, velocity_interp=1))
    assert kpstm_lib.kpstm_create(C.byref(prm), C.byref(vel), C.byref(h)) == 11  # KPSTM_ERR_UNSUPPORTED
    prm = capi.make_params(dict(s.params, velocity_interp=2))
    assert kpstm_lib.kpstm_create(C.byref(prm), C.byref(vel), C.byref(h)) == 1
    del keep


def test_no_cpu_fallback_without_gpu(kpstm_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    s, *_ = load("g1_line_oddns")
    prm = capi.make_params(s.params)
    vel, keep = capi.make_velocity(s.velocity)
    h = C.c_void_p()
    assert kpstm_lib.kpstm_create(C.byref(prm), C.byref(vel), C.byref(h)) == 9  # KPSTM_ERR_NO_DEVICE
    del keep

