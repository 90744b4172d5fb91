"""ctypes binding of the C ABI declared in include/kpstm.h.

This is the binding a Python caller of the reference's kirchhoff() job would
add: the structures mirror kpstm_params /
kpstm_velocity / kpstm_dims field for field, and ``load()`` opens the
in-tree ``libkpstm.so`` built by ``random_gb300.build``.  There is no
fallback: if the library is missing or no GPU is visible the calls fail.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libkpstm.so"

MODE_REFERENCE, MODE_FULL = 0, 1
PREC_FP32, PREC_BF16_KAHAN = 0, 1
OUT_OFFSET_GATHERS, OUT_STACK = 0, 1

STATUS = {
    0: "KPSTM_OK", 1: "KPSTM_ERR_INVALID_ARG", 2: "KPSTM_ERR_CUDA", 3: "KPSTM_ERR_OUT_OF_MEMORY",
    4: "KPSTM_ERR_VELOCITY_ZERO", 5: "KPSTM_ERR_VELOCITY_RANGE", 6: "KPSTM_ERR_GEOMETRY",
    7: "KPSTM_ERR_STATE", 8: "KPSTM_ERR_TIMEOUT", 9: "KPSTM_ERR_NO_DEVICE", 10: "KPSTM_ERR_SEGY",
    11: "KPSTM_ERR_UNSUPPORTED", 12: "KPSTM_ERR_TRANGE", 13: "KPSTM_ERR_TOO_LARGE",
}
NOALLOC_MAX_SAMPLES = 4194304
NOALLOC_MAX_NS = 5600

# kpstm_cg_monitor: int (*)(int32_t iteration, const float *d_model, double resid_k, void *user)
CG_MONITOR = C.CFUNCTYPE(C.c_int, C.c_int32, C.c_void_p, C.c_double, C.c_void_p)


class KpstmParams(C.Structure):
    _fields_ = [
        ("ns", C.c_int32), ("dt", C.c_float),
        ("start_iline", C.c_int32), ("end_iline", C.c_int32),
        ("start_xline", C.c_int32), ("end_xline", C.c_int32),
        ("inc_iline", C.c_double), ("inc_xline", C.c_double),
        ("iline_distance", C.c_double), ("xline_distance", C.c_double),
        ("nh", C.c_int32), ("oh", C.c_double), ("dh", C.c_double),
        ("ox", C.c_double), ("oy", C.c_double), ("angle_e_to_n_deg", C.c_double),
        ("xy_scale", C.c_double),
        ("aperture", C.c_double), ("anti_alias_cutoff", C.c_double),
        ("jobs_x", C.c_int32), ("jobs_y", C.c_int32), ("job_id", C.c_int32),
        ("mode", C.c_int32), ("precision", C.c_int32), ("output", C.c_int32),
        ("aa_max_halfwidth", C.c_int32), ("velocity_interp", C.c_int32), ("reserved", C.c_int32 * 6),
    ]


class KpstmVelocity(C.Structure):
    _fields_ = [
        ("n_iline", C.c_int32), ("n_xline", C.c_int32), ("nsm", C.c_int32),
        ("o_iline", C.c_int32), ("o_xline", C.c_int32), ("d_iline", C.c_int32),
        ("d_xline", C.c_int32), ("dtm", C.c_float), ("vrms", C.c_void_p),
    ]


class KpstmProfile(C.Structure):
    _fields_ = [("image_launches", C.c_int64), ("image_ms", C.c_double), ("prep_ms", C.c_double),
                ("finish_ms", C.c_double), ("other_launches", C.c_int64)]


class KpstmLaunch(C.Structure):
    _fields_ = [("tile_px", C.c_int32), ("samples_per_lane", C.c_int32), ("persistent", C.c_int32),
                ("graph", C.c_int32), ("ctas_per_sm", C.c_int32), ("reserved", C.c_int32 * 3)]


class KpstmDims(C.Structure):
    _fields_ = [
        ("Nx", C.c_int32), ("Ny", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32),
        ("nh", C.c_int32), ("ns", C.c_int32), ("trange_max", C.c_int32),
        ("x0", C.c_int32), ("y0", C.c_int32), ("out_elems", C.c_int64),
    ]


def make_params(p: dict) -> KpstmParams:
    s = KpstmParams()
    for name, _ in KpstmParams._fields_:
        if name == "reserved":
            continue
        if name in p:
            setattr(s, name, p[name])
    if "xy_scale" not in p:
        s.xy_scale = 1.0
    return s


def make_velocity(v) -> tuple[KpstmVelocity, np.ndarray]:
    arr = np.ascontiguousarray(v.vrms, dtype=np.float32)
    s = KpstmVelocity(v.n_iline, v.n_xline, v.nsm, v.o_iline, v.o_xline, v.d_iline, v.d_xline,
                      v.dtm, arr.ctypes.data)
    return s, arr


def oracle_dims(p: dict) -> dict:
    """Slab sizes as main() computes them (Kirchhoff.c:266-300)."""
    Nx = 1 if p["inc_iline"] == 0 else int(math.ceil((p["end_iline"] - p["start_iline"]) / p["inc_iline"]))
    Ny = 1 if p["inc_xline"] == 0 else int(math.ceil((p["end_xline"] - p["start_xline"]) / p["inc_xline"]))
    Nx, Ny = Nx or 1, Ny or 1
    nx = int(math.ceil(1.0 * Nx / p.get("jobs_x", 1))) or 1
    ny = int(math.ceil(1.0 * Ny / p.get("jobs_y", 1))) or 1
    nh = 1 if p.get("output", 0) == OUT_STACK else p["nh"]
    ns = p["ns"]
    return dict(Nx=Nx, Ny=Ny, nx=nx, ny=ny, nh=nh, ns=ns, shape=(nx, ny, nh, ns),
                out_elems=nx * ny * nh * ns)


class KpstmError(RuntimeError):
    def __init__(self, fn: str, status: int):
        super().__init__(f"{fn} failed: {STATUS.get(status, status)}")
        self.status = status


_lib = None
_VOIDP = C.c_void_p


def _sig(lib, name, restype, argtypes):
    f = getattr(lib, name)
    f.restype = restype
    f.argtypes = argtypes
    return f


def load() -> C.CDLL:
    """Open the in-tree library; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise FileNotFoundError(f"{LIB_PATH} not built: run random_gb300.build.build()")
    lib = C.CDLL(str(LIB_PATH))
    i32, i64 = C.c_int32, C.c_int64
    _sig(lib, "kpstm_create", C.c_int, [C.POINTER(KpstmParams), C.POINTER(KpstmVelocity), C.POINTER(_VOIDP)])
    _sig(lib, "kpstm_destroy", None, [_VOIDP])
    _sig(lib, "kpstm_get_dims", C.c_int, [_VOIDP, C.POINTER(KpstmDims)])
    _sig(lib, "kpstm_reset", C.c_int, [_VOIDP])
    _sig(lib, "kpstm_add_traces", C.c_int, [_VOIDP, _VOIDP, _VOIDP, i64])
    _sig(lib, "kpstm_add_segy_block", C.c_int, [_VOIDP, _VOIDP, i64])
    _sig(lib, "kpstm_add_traces_device", C.c_int, [_VOIDP, _VOIDP, _VOIDP, i64])
    _sig(lib, "kpstm_finish", C.c_int, [_VOIDP, _VOIDP, _VOIDP])
    _sig(lib, "kpstm_finish_device", C.c_int, [_VOIDP, _VOIDP, _VOIDP])
    _sig(lib, "kpstm_get_accumulators", C.c_int, [_VOIDP, _VOIDP, _VOIDP])
    _sig(lib, "kpstm_pair_count", C.c_int, [_VOIDP, C.POINTER(i64)])
    _sig(lib, "kpstm_synchronize", C.c_int, [_VOIDP])
    _sig(lib, "kpstm_set_stream", C.c_int, [_VOIDP, _VOIDP])
    _sig(lib, "kpstm_profile_enable", C.c_int, [_VOIDP, C.c_int])
    _sig(lib, "kpstm_profile_read", C.c_int, [_VOIDP, C.POINTER(KpstmProfile)])
    _sig(lib, "kpstm_get_launch", C.c_int, [_VOIDP, C.POINTER(KpstmLaunch)])
    _sig(lib, "kpstm_set_launch", C.c_int, [_VOIDP, C.POINTER(KpstmLaunch)])
    _sig(lib, "kpstm_autotune", C.c_int, [_VOIDP, _VOIDP, _VOIDP, i64, C.POINTER(KpstmLaunch),
                                         C.POINTER(C.c_float)])
    _sig(lib, "kpstm_lsm_geometry", C.c_int, [_VOIDP, _VOIDP, i64])
    _sig(lib, "kpstm_lsm_adjoint", C.c_int, [_VOIDP, _VOIDP, _VOIDP])
    _sig(lib, "kpstm_lsm_forward", C.c_int, [_VOIDP, _VOIDP, _VOIDP])
    _sig(lib, "kpstm_lsm_cg", C.c_int, [_VOIDP, _VOIDP, C.c_int32, _VOIDP, _VOIDP])
    _sig(lib, "kpstm_lsm_cg_ex", C.c_int, [_VOIDP, _VOIDP, C.c_int32, _VOIDP, _VOIDP, CG_MONITOR, _VOIDP])
    _sig(lib, "kpstm_lsm_pair_count", C.c_int, [_VOIDP, C.POINTER(i64)])
    _sig(lib, "kpstm_finish_noalloc", C.c_int, [C.POINTER(KpstmParams), _VOIDP, _VOIDP, _VOIDP, _VOIDP])
    _sig(lib, "kpstm_aliasfilter", C.c_int, [i32, C.c_float, C.c_double, C.c_double, C.c_double,
                                            C.POINTER(i32), _VOIDP])
    _sig(lib, "kpstm_ibm_to_ieee", C.c_int, [_VOIDP, _VOIDP, i64])
    _sig(lib, "kpstm_segy_info", C.c_int, [_VOIDP, i64, C.POINTER(i32), C.POINTER(C.c_float),
                                          C.POINTER(i64)])
    _sig(lib, "kpstm_write_su", C.c_int, [_VOIDP, _VOIDP, _VOIDP, i64])
    _sig(lib, "kpstm_segy_front_headers", C.c_int, [C.POINTER(KpstmParams), _VOIDP, i64])
    _sig(lib, "kpstm_velocity_from_segy", C.c_int, [_VOIDP, i64, i32, i32, i32, i32, i32, i32, _VOIDP, i64])
    _sig(lib, "kpstm_debug_wait_limit", C.c_int, [_VOIDP, C.c_uint32])
    _sig(lib, "kpstm_debug_fail_alloc", C.c_int, [C.c_int32])
    _sig(lib, "kpstm_debug_trace_cull", C.c_int, [_VOIDP, C.c_int32])
    _sig(lib, "kpstm_strerror", C.c_char_p, [C.c_int])
    _sig(lib, "kpstm_abi_version", C.c_int, [])
    _lib = lib
    return lib


def check(fn: str, status: int) -> None:
    if status != 0:
        raise KpstmError(fn, status)
