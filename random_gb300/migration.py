"""Python front end of libkpstm (ctypes over include/kpstm.h).

``Migration`` is one imaging job - the reference's ``kirchhoff(job_id)``
(Kirchhoff.c:1104) with its set-up (main :263-331): create it with the
job's parameters and v_rms model, feed trace blocks in file order (one
``ntblock`` read of Kirchhoff.c:1276-1290 per call), then ``finish()``
returns the finished image [nx, ny, nh, ns] as the reference writes it
(:1440-1479).  Every call goes to the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi, segy


class Migration:
    def __init__(self, params: dict, velocity):
        self._lib = capi.load()
        self.params = dict(params)
        prm = capi.make_params(self.params)
        vel, keep = capi.make_velocity(velocity)
        h = C.c_void_p()
        capi.check("kpstm_create", self._lib.kpstm_create(C.byref(prm), C.byref(vel), C.byref(h)))
        del keep
        self._h = h
        d = capi.KpstmDims()
        capi.check("kpstm_get_dims", self._lib.kpstm_get_dims(self._h, C.byref(d)))
        self.dims = {f: getattr(d, f) for f, _ in capi.KpstmDims._fields_}
        self.shape = (d.nx, d.ny, d.nh, d.ns)

    # -- lifetime -------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.kpstm_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- traces ---------------------------------------------------------------
    def add_traces(self, headers: np.ndarray, samples: np.ndarray, headers_are_be: bool = False) -> None:
        """headers: [ntr, 60] int32 header words (host order unless
        ``headers_are_be``); samples: [ntr, ns] float32."""
        hdr = np.ascontiguousarray(headers if headers_are_be else segy.headers_be(headers), dtype=np.int32)
        smp = np.ascontiguousarray(samples, dtype=np.float32)
        ntr = smp.shape[0]
        if hdr.shape != (ntr, 60) or smp.shape[1] != self.shape[3]:
            raise ValueError("headers/samples shape mismatch")
        capi.check("kpstm_add_traces",
                   self._lib.kpstm_add_traces(self._h, hdr.ctypes.data, smp.ctypes.data, ntr))

    def add_traces_ptr(self, hdr_be_ptr: int, samples_ptr: int, ntr: int) -> None:
        """Host pointers (e.g. pinned buffers) to BE header words and samples."""
        capi.check("kpstm_add_traces", self._lib.kpstm_add_traces(self._h, hdr_be_ptr, samples_ptr, ntr))

    def add_traces_device(self, d_hdr_be: int, d_samples: int, ntr: int) -> None:
        """Device pointers; the work is queued on the context's stream."""
        capi.check("kpstm_add_traces_device",
                   self._lib.kpstm_add_traces_device(self._h, d_hdr_be, d_samples, ntr))

    def add_segy_block(self, records: np.ndarray) -> None:
        """records: uint8 [ntr, 240 + 4*ns] raw SEG-Y trace records (IBM floats)."""
        rec = np.ascontiguousarray(records, dtype=np.uint8)
        capi.check("kpstm_add_segy_block", self._lib.kpstm_add_segy_block(self._h, rec.ctypes.data, rec.shape[0]))

    # -- results --------------------------------------------------------------
    def finish(self, want_fold: bool = False):
        out = np.empty(self.shape, np.float32)
        fold = np.empty(self.shape, np.float32) if want_fold else None
        capi.check("kpstm_finish", self._lib.kpstm_finish(
            self._h, out.ctypes.data, None if fold is None else fold.ctypes.data))
        return (out, fold) if want_fold else out

    def finish_ptr(self, out_ptr: int, fold_ptr: int | None = None) -> None:
        capi.check("kpstm_finish", self._lib.kpstm_finish(self._h, out_ptr, fold_ptr))

    def finish_device(self, d_out: int, d_fold: int | None = None) -> None:
        capi.check("kpstm_finish_device", self._lib.kpstm_finish_device(self._h, d_out, d_fold))

    def accumulators(self):
        km = np.empty(self.shape, np.float32)
        fold = np.empty(self.shape, np.float32)
        capi.check("kpstm_get_accumulators",
                   self._lib.kpstm_get_accumulators(self._h, km.ctypes.data, fold.ctypes.data))
        return km, fold

    def pairs(self) -> int:
        v = C.c_int64()
        capi.check("kpstm_pair_count", self._lib.kpstm_pair_count(self._h, C.byref(v)))
        return v.value

    def set_stream(self, stream_handle: int | None) -> None:
        capi.check("kpstm_set_stream", self._lib.kpstm_set_stream(self._h, stream_handle))

    def profile(self, enable: bool = True) -> None:
        capi.check("kpstm_profile_enable", self._lib.kpstm_profile_enable(self._h, int(enable)))

    def profile_read(self) -> dict:
        pr = capi.KpstmProfile()
        capi.check("kpstm_profile_read", self._lib.kpstm_profile_read(self._h, C.byref(pr)))
        return {f: getattr(pr, f) for f, _ in capi.KpstmProfile._fields_}

    # -- launch configuration of the imaging kernel ------------------------
    def launch_config(self) -> dict:
        cfg = capi.KpstmLaunch()
        capi.check("kpstm_get_launch", self._lib.kpstm_get_launch(self._h, C.byref(cfg)))
        return {f: getattr(cfg, f) for f, _ in capi.KpstmLaunch._fields_ if f != "reserved"}

    def set_launch(self, tile_px: int = 0, samples_per_lane: int = 0, persistent: int = 0, graph: int = 0,
                   ctas_per_sm: int = 0) -> None:
        """Imaging work split (kpstm_set_launch); results are identical for every choice."""
        cfg = capi.KpstmLaunch(tile_px=tile_px, samples_per_lane=samples_per_lane, persistent=persistent,
                               graph=graph, ctas_per_sm=ctas_per_sm)
        capi.check("kpstm_set_launch", self._lib.kpstm_set_launch(self._h, C.byref(cfg)))

    def autotune(self, d_hdr_be: int, d_samples: int, ntr: int) -> tuple[dict, float]:
        """kpstm_autotune on a device block; returns (chosen configuration, its block time in ms)."""
        cfg = capi.KpstmLaunch()
        ms = C.c_float()
        capi.check("kpstm_autotune", self._lib.kpstm_autotune(self._h, d_hdr_be, d_samples, ntr, C.byref(cfg),
                                                               C.byref(ms)))
        return {f: getattr(cfg, f) for f, _ in capi.KpstmLaunch._fields_ if f != "reserved"}, ms.value

    # -- least-squares migration (device pointers) ----------------------------
    def lsm_geometry(self, headers: np.ndarray, headers_are_be: bool = False) -> None:
        hdr = np.ascontiguousarray(headers if headers_are_be else segy.headers_be(headers), dtype=np.int32)
        capi.check("kpstm_lsm_geometry", self._lib.kpstm_lsm_geometry(self._h, hdr.ctypes.data, hdr.shape[0]))

    def lsm_adjoint(self, d_data: int, d_model: int) -> None:
        """d_model = L^T d_data (migration)."""
        capi.check("kpstm_lsm_adjoint", self._lib.kpstm_lsm_adjoint(self._h, d_data, d_model))

    def lsm_forward(self, d_model: int, d_data: int) -> None:
        """d_data = L d_model (demigration)."""
        capi.check("kpstm_lsm_forward", self._lib.kpstm_lsm_forward(self._h, d_model, d_data))

    def lsm_pairs(self) -> int:
        """Pairs of one operator application (counted by the last lsm_adjoint)."""
        v = C.c_int64()
        capi.check("kpstm_lsm_pair_count", self._lib.kpstm_lsm_pair_count(self._h, C.byref(v)))
        return v.value

    def lsm_cg(self, d_data: int, niter: int, d_model: int, monitor=None) -> np.ndarray:
        """CGLS from m = 0 (kpstm_lsm_cg_ex).  ``monitor(k, d_model_ptr, resid_k)``,
        if given, runs after iteration k has updated the model; a truthy
        return ends the solve there.  Returns the residual norms reached."""
        resid = np.full(niter + 1, np.nan, np.float64)
        if monitor is None:
            capi.check("kpstm_lsm_cg", self._lib.kpstm_lsm_cg(self._h, d_data, niter, d_model, resid.ctypes.data))
            return resid
        err = []

        def _cb(k, ptr, res, _user):
            try:
                return 1 if monitor(int(k), int(ptr or 0), float(res)) else 0
            except BaseException as e:  # a Python error must not unwind through C
                err.append(e)
                return 1

        cb = capi.CG_MONITOR(_cb)
        st = self._lib.kpstm_lsm_cg_ex(self._h, d_data, niter, d_model, resid.ctypes.data, cb, None)
        if err:
            raise err[0]
        capi.check("kpstm_lsm_cg_ex", st)
        return resid[~np.isnan(resid)]

    def synchronize(self) -> None:
        capi.check("kpstm_synchronize", self._lib.kpstm_synchronize(self._h))

    def reset(self) -> None:
        capi.check("kpstm_reset", self._lib.kpstm_reset(self._h))

    def write_su(self, image: np.ndarray) -> bytes:
        ns = self.shape[3]
        n = self.shape[0] * self.shape[1] * self.shape[2]
        buf = np.empty(n * (240 + 4 * ns), np.uint8)
        img = np.ascontiguousarray(image, np.float32)
        capi.check("kpstm_write_su", self._lib.kpstm_write_su(self._h, img.ctypes.data, buf.ctypes.data, buf.size))
        return buf.tobytes()


def migrate(survey, params: dict | None = None, block: int = 50000, want_acc: bool = False):
    """Image a synth.Survey in blocks of ``block`` traces (the reference's
    ntblock).  Returns dict(image, fold, km?, pairs)."""
    p = dict(survey.params)
    if params:
        p.update(params)
    with Migration(p, survey.velocity) as m:
        for b0 in range(0, survey.ntr, block):
            m.add_traces(survey.headers[b0:b0 + block], survey.samples[b0:b0 + block])
        image, fold = m.finish(want_fold=True)
        out = dict(image=image, fold=fold, pairs=m.pairs())
        if want_acc:
            out["km"], out["fold_acc"] = m.accumulators()
        return out


def segy_front_headers(params: dict) -> bytes:
    """The 3600 front-header bytes of the output SEG-Y file
    (kpstm_segy_front_headers; no device needed)."""
    lib = capi.load()
    prm = capi.make_params(params)
    buf = np.zeros(3600, np.uint8)
    capi.check("kpstm_segy_front_headers", lib.kpstm_segy_front_headers(C.byref(prm), buf.ctypes.data, buf.size))
    return buf.tobytes()


def combine_su(out_path, params: dict, slab_files) -> None:
    """The reference's combine step (Kirchhoff.c:821-874): front headers,
    then each slab's SU records (image<job>.su) in job order, into one file."""
    with open(out_path, "wb") as out:
        out.write(segy_front_headers(params))
        for f in slab_files:
            with open(f, "rb") as src:
                while True:
                    chunk = src.read(1 << 24)
                    if not chunk:
                        break
                    out.write(chunk)


def velocity_from_segy(file_bytes: bytes, n_iline: int, n_xline: int, o_iline: int, o_xline: int, d_iline: int,
                       d_xline: int):
    """build_vel_model from a velocity SEG-Y file image: returns (vrms
    [n_iline, n_xline, nsm] float32, nsm, dtm) via kpstm_velocity_from_segy."""
    lib = capi.load()
    raw = np.frombuffer(file_bytes, np.uint8)
    ns, dt, ntr = C.c_int32(), C.c_float(), C.c_int64()
    capi.check("kpstm_segy_info", lib.kpstm_segy_info(raw.ctypes.data, raw.size, C.byref(ns), C.byref(dt),
                                                      C.byref(ntr)))
    out = np.zeros((n_iline, n_xline, ns.value), np.float32)
    capi.check("kpstm_velocity_from_segy",
               lib.kpstm_velocity_from_segy(raw.ctypes.data, raw.size, n_iline, n_xline, o_iline, o_xline, d_iline,
                                            d_xline, out.ctypes.data, out.size))
    return out, ns.value, dt.value
