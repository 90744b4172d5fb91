"""ctypes wrapper of the C oracle (kpstm_oracle.c) - TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, as the checker.  ``build()`` compiles the oracle library into
``oracle/_build`` (gcc, -O2 -ffp-contract=off, no machine-specific flags so
that x86-64 and aarch64 compute identical results).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libkpstm_oracle.so"
SOURCES = [HERE / "kpstm_oracle.c", HERE / "shim" / "fftw_shim.c"]


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    newest = max(s.stat().st_mtime for s in SOURCES + [HERE / "kpstm_oracle.h"])
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_suffix(f".so.{os.getpid()}")
    cmd = ["gcc", "-std=gnu17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
           f"-I{HERE}", *map(str, SOURCES), "-lm", "-o", str(tmp)]
    subprocess.run(cmd, check=True, capture_output=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C")
        _lib.ko_kirchhoff.restype = C.c_int
        _lib.ko_kirchhoff.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                      C.POINTER(C.c_int64)]
        _lib.ko_finish.restype = C.c_int
        _lib.ko_finish.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.ko_aliasfilter.restype = C.c_int
        _lib.ko_aliasfilter.argtypes = [C.c_int, C.c_float, C.c_double, C.c_double, C.c_double,
                                        C.POINTER(C.c_int), C.c_void_p]
        _lib.ko_kirchhoff64.restype = C.c_int
        _lib.ko_kirchhoff64.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                        C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.ko_lsm_apply.restype = C.c_int
        _lib.ko_lsm_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p,
                                      C.c_void_p]
        _lib.ko_prep_trace.restype = None
        _lib.ko_prep_trace.argtypes = [C.c_int, C.c_int, C.c_float, f32p, f32p, f32p]
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def aliasfilter(ns: int, dt: float, il_dist: float, xl_dist: float, cutoff: float):
    tm = C.c_int()
    aa = np.zeros(ns, np.float32)
    st = lib().ko_aliasfilter(ns, dt, il_dist, xl_dist, cutoff, C.byref(tm), _ptr(aa))
    if st:
        raise RuntimeError(f"ko_aliasfilter: status {st}")
    return tm.value, aa


def prep_trace(trace: np.ndarray, t2: np.ndarray, tm: int, dt: float) -> np.ndarray:
    ns = trace.size
    out = np.zeros(ns + 2 * tm, np.float32)
    lib().ko_prep_trace(ns, tm, dt, np.ascontiguousarray(t2, np.float32),
                        np.ascontiguousarray(trace, np.float32), out)
    return out


def kirchhoff(survey, params: dict | None = None, nthreads: int = 0, want_acc: bool = True):
    """Run the oracle job for a synth.Survey.  Returns dict(image, km, fold, pairs)."""
    from random_gb300 import capi, segy  # struct layouts only; no library calls
    p = dict(survey.params)
    if params:
        p.update(params)
    prm = capi.make_params(p)
    vel, _keep = capi.make_velocity(survey.velocity)
    dims = capi.oracle_dims(p)
    nimg = dims["out_elems"]
    image = np.zeros(nimg, np.float32)
    km = np.zeros(nimg, np.float32) if want_acc else None
    fold = np.zeros(nimg, np.float32) if want_acc else None
    hdr = np.ascontiguousarray(segy.headers_be(survey.headers))
    smp = np.ascontiguousarray(survey.samples, np.float32)
    pairs = C.c_int64()
    st = lib().ko_kirchhoff(C.addressof(prm), C.addressof(vel), _ptr(hdr), _ptr(smp), survey.ntr,
                            _ptr(km), _ptr(fold), _ptr(image), int(nthreads), C.byref(pairs))
    if st:
        raise RuntimeError(f"ko_kirchhoff: status {st}")
    shape = dims["shape"]
    return dict(image=image.reshape(shape), km=None if km is None else km.reshape(shape),
                fold=None if fold is None else fold.reshape(shape), pairs=pairs.value)


def lsm_apply(survey, direction: int, vec: np.ndarray, params: dict | None = None) -> np.ndarray:
    """Full-mode least-squares operators in double: direction 0 = L^T
    (data [ntr, ns] -> model [nx, ny, nh, ns]), 1 = L (model -> data)."""
    from random_gb300 import capi, segy
    p = dict(survey.params)
    if params:
        p.update(params)
    prm = capi.make_params(p)
    vel, _keep = capi.make_velocity(survey.velocity)
    dims = capi.oracle_dims(p)
    hdr = np.ascontiguousarray(segy.headers_be(survey.headers))
    src = np.ascontiguousarray(vec, dtype=np.float64)
    out = np.zeros(dims["shape"] if direction == 0 else (survey.ntr, survey.ns), np.float64)
    st = lib().ko_lsm_apply(C.addressof(prm), C.addressof(vel), hdr.ctypes.data, survey.ntr, direction,
                            src.ctypes.data, out.ctypes.data)
    if st:
        raise RuntimeError(f"ko_lsm_apply: status {st}")
    return out


def kirchhoff64(survey, params: dict | None = None):
    """FP64 oracle job: dict(image, km, fold) as float64 [nx, ny, nh, ns]."""
    from random_gb300 import capi, segy
    p = dict(survey.params)
    if params:
        p.update(params)
    prm = capi.make_params(p)
    vel, _keep = capi.make_velocity(survey.velocity)
    dims = capi.oracle_dims(p)
    out = {k: np.zeros(dims["shape"], np.float64) for k in ("image", "km", "fold")}
    hdr = np.ascontiguousarray(segy.headers_be(survey.headers))
    smp = np.ascontiguousarray(survey.samples, np.float32)
    st = lib().ko_kirchhoff64(C.addressof(prm), C.addressof(vel), hdr.ctypes.data, smp.ctypes.data, survey.ntr,
                              out["km"].ctypes.data, out["fold"].ctypes.data, out["image"].ctypes.data)
    if st:
        raise RuntimeError(f"ko_kirchhoff64: status {st}")
    return out


def cgls(survey, d: np.ndarray, niter: int, params: dict | None = None):
    """FP64 CGLS on min |L m - d|^2 from m = 0 with the oracle operators
    (lsm_apply), the same recurrence as the library's kpstm_lsm_cg: r = d,
    s = L^T r, p = s; per iteration q = L p, alpha = |s|^2/|q|^2,
    m += alpha p, r -= alpha q, s = L^T r, beta = |s_new|^2/|s|^2,
    p = s + beta p (the last iteration stops after the update of m and r).
    Returns (iterates [niter] of float64 models, residual norms [niter + 1])."""
    d = np.asarray(d, np.float64)
    r = d.copy()
    s_ = lsm_apply(survey, 0, r, params)
    p = s_.copy()
    x = np.zeros_like(s_)
    gamma = float(np.vdot(s_, s_))
    res, xs = [float(np.linalg.norm(r))], []
    for it in range(niter):
        q = lsm_apply(survey, 1, p, params)
        qq = float(np.vdot(q, q))
        alpha = gamma / qq if qq > 0 else 0.0
        x += alpha * p
        r -= alpha * q
        res.append(float(np.linalg.norm(r)))
        xs.append(x.copy())
        if it + 1 == niter:
            break
        s_ = lsm_apply(survey, 0, r, params)
        gnew = float(np.vdot(s_, s_))
        p = s_ + (gnew / gamma if gamma > 0 else 0.0) * p
        gamma = gnew
    return xs, np.array(res)
