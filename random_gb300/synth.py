"""Seeded synthetic surveys for the migration workloads.

The reference ships no data (its Ghana field files are absent), so every
workload is synthesised from a written description: geometry, sampling,
events (Ricker wavelets on double-square-root or mirror-source traveltimes),
v_rms model and noise.  Each survey carries the kpstm_params values and the
matching compile-time configuration of the reference (Kirchhoff.c:17-65),
so that the reference, the oracle and the GPU library image the same thing.

Coordinates are integers in the headers because the reference truncates
header coordinates to int (Kirchhoff.c:1297, 1302).  The 2-D line survey
(12.5 m CMP spacing) is therefore written in half-metre units: every length,
the aperture and the velocities are doubled, which leaves all traveltimes
(and, since the reference's triangle half-width is fixed at 2 samples,
every imaged value) unchanged.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import segy


@dataclass
class Velocity:
    n_iline: int
    n_xline: int
    nsm: int
    o_iline: int
    o_xline: int
    d_iline: int
    d_xline: int
    dtm: float
    vrms: np.ndarray  # [n_iline, n_xline, nsm] float32

    @property
    def dtm_us(self) -> int:
        return int(round(self.dtm * 1e6))


@dataclass
class Survey:
    name: str
    params: dict
    velocity: Velocity
    headers: np.ndarray          # [ntr, 60] int32, host order
    samples: np.ndarray          # [ntr, ns] float32 (IBM-representable)
    info: dict = field(default_factory=dict)

    @property
    def ntr(self) -> int:
        return self.headers.shape[0]

    @property
    def ns(self) -> int:
        return int(self.params["ns"])

    @property
    def dt_us(self) -> int:
        return int(round(self.params["dt"] * 1e6))

    def ref_config(self, jobs_x: int = 1, jobs_y: int = 1, ntblock: int | None = None) -> dict:
        """Values for the reference's #define block (Kirchhoff.c:17-65)."""
        p, v = self.params, self.velocity
        return dict(
            NVel_ilines=v.n_iline, NVel_xlines=v.n_xline, dVel_ilines=v.d_iline,
            dVel_xlines=v.d_xline, oVel_ilines=v.o_iline, oVel_xlines=v.o_xline,
            Startiline=p["start_iline"], Endiline=p["end_iline"],
            Startxline=p["start_xline"], Endxline=p["end_xline"],
            INCiline=p["inc_iline"], INCxline=p["inc_xline"], dh=p["dh"], nh=p["nh"],
            oh=p["oh"], ox=p["ox"], oy=p["oy"], angleEtoN=p["angle_e_to_n_deg"],
            iline_distance=p["iline_distance"], xline_distance=p["xline_distance"],
            aperture=p["aperture"], anti_alias_cutoff=p["anti_alias_cutoff"],
            ntblock=ntblock or max(1, self.ntr), number_mpi_jobsX=jobs_x,
            number_mpi_jobsY=jobs_y)

    def write_files(self, data_path, vel_path) -> None:
        segy.write_segy(data_path, self.headers, self.samples)
        v = self.velocity
        vh = segy.velocity_headers(v.n_iline, v.n_xline, v.o_iline, v.o_xline,
                                   v.d_iline, v.d_xline, v.nsm, v.dtm_us)
        segy.write_segy(vel_path, vh, v.vrms.reshape(v.n_iline * v.n_xline, v.nsm))


def default_params(**kw) -> dict:
    p = dict(ns=0, dt=0.0, start_iline=0, end_iline=0, start_xline=0, end_xline=0,
             inc_iline=1.0, inc_xline=1.0, iline_distance=25.0, xline_distance=25.0,
             nh=1, oh=0.0, dh=1.0, ox=0.0, oy=0.0, angle_e_to_n_deg=0.0, xy_scale=1.0,
             aperture=3000.0, anti_alias_cutoff=50.0, jobs_x=1, jobs_y=1, job_id=0,
             mode=0, precision=0, output=0, aa_max_halfwidth=0)
    p.update(kw)
    return p


def ricker(tau: np.ndarray, f: float) -> np.ndarray:
    a = (math.pi * f * tau) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)


def _add_events(samples: np.ndarray, t_event: np.ndarray, amp: np.ndarray, dt: float,
                f: float, half_width: int) -> None:
    """samples[i, :] += amp[i, e] * ricker(t - t_event[i, e]) over a window."""
    ntr, ns = samples.shape
    k = np.arange(-half_width, half_width + 1)
    for e in range(t_event.shape[1]):
        te = t_event[:, e]
        c = np.floor(te / dt).astype(np.int64)
        idx = c[:, None] + k[None, :]
        ok = (idx >= 0) & (idx < ns)
        w = ricker(idx * dt - te[:, None], f) * amp[:, e:e + 1]
        rows = np.broadcast_to(np.arange(ntr)[:, None], idx.shape)
        np.add.at(samples, (rows[ok], idx[ok]), w[ok])


def line2d(n_cmp: int = 200, n_off: int = 48, ns: int = 1001, dt: float = 0.004,
           n_scat: int = 20, snr_db: float = 20.0, seed: int = 1,
           aperture_m: float = 1500.0, aa_cutoff: float = 1.0e6,
           name: str = "line2d") -> Survey:
    """2-D line: n_cmp CMPs at 12.5 m x n_off offsets (0, 50, ... m), point
    scatterers with 25 Hz Ricker diffraction hyperbolae, v_rms = 1500 +
    600*t0 m/s, Gaussian noise at ``snr_db``; image n_cmp columns x n_off
    classes x ns.  Anti-alias "off" is a cutoff far above Nyquist: the
    reference's [1,2,1] triangle taps are intrinsic to its operator
    (Kirchhoff.c:1391-1392), only its low-pass can be switched off.

    Half-metre units (see module docstring): CMP spacing 25, offsets 100.
    """
    rng = np.random.default_rng(seed)
    u = 2.0                                     # units per metre
    d_cmp = 12.5 * u                            # 25 units
    start_il = 96                               # IX = start_il * 25 = 2400 units
    x0 = start_il * d_cmp
    y_line = 4 * d_cmp                          # xline 4
    cmp_x = x0 + d_cmp * np.arange(n_cmp)
    half = 25.0 * u * np.arange(n_off)          # half-offsets (units)
    mx = np.repeat(cmp_x, n_off)
    hh = np.tile(half, n_cmp)
    sx = (mx - hh).astype(np.int64)
    gx = (mx + hh).astype(np.int64)
    if sx.min() < 0:
        raise ValueError("survey extends below coordinate 0")
    sy = np.full_like(sx, int(y_line))
    gy = sy.copy()
    ntr = sx.size

    # scatterers
    px = rng.uniform(cmp_x[0], cmp_x[-1], n_scat)
    pt0 = rng.uniform(0.4, 3.6, n_scat)
    pamp = rng.uniform(0.5, 1.0, n_scat)
    pv = (1500.0 + 600.0 * pt0) * u
    ts = np.sqrt(0.25 * pt0[None, :] ** 2 + ((sx[:, None] - px[None, :]) / pv[None, :]) ** 2)
    tg = np.sqrt(0.25 * pt0[None, :] ** 2 + ((gx[:, None] - px[None, :]) / pv[None, :]) ** 2)
    samples = np.zeros((ntr, ns), dtype=np.float64)
    _add_events(samples, ts + tg, np.broadcast_to(pamp, (ntr, n_scat)).copy(), dt, 25.0,
                half_width=int(math.ceil(0.08 / dt)))
    sig_rms = float(np.sqrt(np.mean(samples ** 2)))
    if snr_db is not None and sig_rms > 0:
        samples += rng.normal(0.0, sig_rms / 10.0 ** (snr_db / 20.0), samples.shape)
    samples = segy.ibm_roundtrip(samples.astype(np.float32))
    hdr = segy.trace_headers(sx, sy, gx, gy, ns, int(round(dt * 1e6)),
                             {segy.W_OFFSET: (gx - sx)})

    nsm = ns
    t0 = np.arange(nsm) * dt
    vt = ((1500.0 + 600.0 * t0) * u).astype(np.float32)
    vel = Velocity(n_iline=n_cmp, n_xline=1, nsm=nsm, o_iline=start_il, o_xline=4,
                   d_iline=1, d_xline=1, dtm=dt,
                   vrms=segy.ibm_roundtrip(np.broadcast_to(vt, (n_cmp, 1, nsm)).copy()))
    params = default_params(
        ns=ns, dt=float(np.float32(int(round(dt * 1e6)) / 1e6)),
        start_iline=start_il, end_iline=start_il + n_cmp, start_xline=4, end_xline=4,
        iline_distance=d_cmp, xline_distance=d_cmp, nh=n_off, oh=0.0,
        dh=50.0 * u, aperture=aperture_m * u, anti_alias_cutoff=aa_cutoff)
    # oh = -dh/2 centres each class on its nominal offset: class k holds
    # offsets in [100k - 50, 100k + 50) units, so no offset sits on a class edge.
    params["oh"] = -0.5 * params["dh"]
    info = dict(units_per_metre=u, scatterers=np.stack([px, pt0, pamp], 1), seed=seed)
    return Survey(name, params, vel, hdr, samples, info)


def vrms_3d(x: np.ndarray, t0: np.ndarray, v0: float, vt: float, va: float,
            lam: float) -> np.ndarray:
    """v_rms(x, t0) = v0 + vt*t0 + va*sin(2*pi*x/lam)."""
    return v0 + vt * t0 + va * np.sin(2.0 * math.pi * x / lam)


@dataclass
class Patch3DModel:
    """Geometry, events and v_rms of a 3-D patch survey; samples are
    synthesised separately (numpy here, torch on a GPU for full-size runs)."""
    survey: Survey                       # headers/params/velocity; samples empty
    coords: np.ndarray                   # [ntr, 4] float64 grid-frame sx, sy, gx, gy
    refl: dict                           # t0, vk, z0, nrm [n, 3], amp, xc, yc
    diff: dict                           # x, y, t0, v, amp
    freq: float
    half_width: int


def patch3d_model(ntr: int, ns: int = 1501, dt: float = 0.002, nx: int = 400, ny: int = 400,
                  bin_m: float = 25.0, max_offset: float = 4000.0, n_refl: int = 8,
                  n_diff: int = 200, freq: float = 30.0, aperture: float = 3000.0,
                  aa_cutoff: float = 100.0, seed: int = 2, mode: int = 1, output: int = 1,
                  nh: int = 1, oh: float = 0.0, dh: float = 1.0e9, offsets=None,
                  v_law=(1600.0, 500.0, 100.0, 8000.0), name: str = "patch3d",
                  trace_slice: slice | None = None, rotate_deg: float = 0.0,
                  origin=(0.0, 0.0), x_shift: float = 0.0) -> Patch3DModel:
    """3-D patch: midpoints uniform over nx*bin x ny*bin metres, offsets
    U(0, max_offset) (or the given array), azimuths U(0, 2 pi); 30 Hz Ricker
    events from ``n_refl`` planar dipping reflectors (dips U(0, 30 deg),
    mirror-source traveltimes in a constant velocity per reflector) plus
    ``n_diff`` point diffractors (DSR traveltimes); smooth v_rms(x, t0) =
    v0 + vt*t0 + va*sin(2 pi x / lam).  Image nx x ny x ns at ``bin_m``.
    ``trace_slice`` keeps only those traces (same seeded survey).
    ``rotate_deg``/``origin`` place the survey in world coordinates the way
    the reference undoes it (Kirchhoff.c:1297-1304): grid (u, v) maps to
    x = ox + cos(a) u - sin(a) v, y = oy + sin(a) u + cos(a) v.
    ``x_shift`` moves the whole survey and image along x (one slab per
    rank in multi-GPU runs)."""
    rng = np.random.default_rng(seed)
    start = int(math.ceil(max_offset / 2.0 / bin_m)) + 4
    start += int(round(x_shift / bin_m))
    x0 = start * bin_m
    y0 = (int(math.ceil(max_offset / 2.0 / bin_m)) + 4) * bin_m
    start_y = int(round(y0 / bin_m))
    W, H = nx * bin_m, ny * bin_m
    mxs = rng.uniform(x0, x0 + W, ntr)
    mys = rng.uniform(y0, y0 + H, ntr)
    off = rng.uniform(0.0, max_offset, ntr) if offsets is None else np.asarray(offsets, float)
    az = rng.uniform(0.0, 2.0 * math.pi, ntr)
    v0, vt, va, lam = v_law
    r_t0 = rng.uniform(0.4, 0.8 * (ns - 1) * dt, n_refl)
    r_dip = np.radians(rng.uniform(0.0, 30.0, n_refl))
    r_az = rng.uniform(0.0, 2.0 * math.pi, n_refl)
    r_amp = rng.uniform(0.5, 1.0, n_refl) * rng.choice([-1.0, 1.0], n_refl)
    d_x = rng.uniform(x0, x0 + W, n_diff)
    d_y = rng.uniform(y0, y0 + H, n_diff)
    d_t0 = rng.uniform(0.4, 0.9 * (ns - 1) * dt, n_diff)
    d_amp = rng.uniform(0.5, 1.0, n_diff)
    if trace_slice is not None:
        mxs, mys, off, az = mxs[trace_slice], mys[trace_slice], off[trace_slice], az[trace_slice]
    h = 0.5 * off
    sx = np.rint(mxs - h * np.cos(az)).astype(np.int64)
    sy = np.rint(mys - h * np.sin(az)).astype(np.int64)
    gx = np.rint(mxs + h * np.cos(az)).astype(np.int64)
    gy = np.rint(mys + h * np.sin(az)).astype(np.int64)
    if rotate_deg != 0.0 or origin != (0.0, 0.0):
        ca, sa = math.cos(math.radians(rotate_deg)), math.sin(math.radians(rotate_deg))
        wx = lambda u, v: np.rint(origin[0] + ca * u - sa * v).astype(np.int64)
        wy = lambda u, v: np.rint(origin[1] + sa * u + ca * v).astype(np.int64)
        hsx, hsy, hgx, hgy = wx(sx, sy), wy(sx, sy), wx(gx, gy), wy(gx, gy)
    else:
        hsx, hsy, hgx, hgy = sx, sy, gx, gy
    if min(hsx.min(), hsy.min(), hgx.min(), hgy.min()) < 0:
        raise ValueError("survey extends below coordinate 0")
    xc, yc = x0 + 0.5 * W, y0 + 0.5 * H
    vk = v0 + vt * r_t0
    nrm = np.stack([np.sin(r_dip) * np.cos(r_az), np.sin(r_dip) * np.sin(r_az), np.cos(r_dip)], 1)
    refl = dict(t0=r_t0, vk=vk, z0=0.5 * vk * r_t0, nrm=nrm, amp=r_amp, xc=xc, yc=yc)
    diff = dict(x=d_x, y=d_y, t0=d_t0, v=vrms_3d(d_x, d_t0, v0, vt, va, lam), amp=d_amp)
    hdr = segy.trace_headers(hsx, hsy, hgx, hgy, ns, int(round(dt * 1e6)))
    t0 = np.arange(ns) * dt
    xs = (start + np.arange(nx)) * bin_m
    vg = vrms_3d(xs[:, None], t0[None, :], v0, vt, va, lam).astype(np.float32)
    vel = Velocity(n_iline=nx, n_xline=1, nsm=ns, o_iline=start, o_xline=start_y, d_iline=1,
                   d_xline=1000000, dtm=dt, vrms=segy.ibm_roundtrip(vg[:, None, :].copy()))
    params = default_params(
        ns=ns, dt=float(np.float32(int(round(dt * 1e6)) / 1e6)), start_iline=start,
        end_iline=start + nx, start_xline=start_y, end_xline=start_y + ny,
        iline_distance=bin_m, xline_distance=bin_m, nh=nh, oh=oh, dh=dh, aperture=aperture,
        anti_alias_cutoff=aa_cutoff, mode=mode, output=output, ox=float(origin[0]),
        oy=float(origin[1]), angle_e_to_n_deg=float(rotate_deg))
    info = dict(seed=seed, x0=x0, y0=y0)
    sv = Survey(name, params, vel, hdr, np.zeros((0, ns), np.float32), info)
    coords = np.stack([sx, sy, gx, gy], 1).astype(np.float64)
    return Patch3DModel(sv, coords, refl, diff, freq, int(math.ceil(0.06 / dt)))


def _event_times(xp, c, refl, diff):
    """Traveltimes [ntr, n_events] of all events for grid coords c [ntr, 4]
    (xp = numpy or torch)."""
    sx, sy, gx, gy = c[:, 0], c[:, 1], c[:, 2], c[:, 3]
    cols = []
    for k in range(len(refl["t0"])):
        n0, n1, n2 = (float(v) for v in refl["nrm"][k])
        dist_s = n2 * float(refl["z0"][k]) - (n0 * (sx - refl["xc"]) + n1 * (sy - refl["yc"]))
        mx_ = sx + 2.0 * dist_s * n0
        my_ = sy + 2.0 * dist_s * n1
        mz_ = 2.0 * dist_s * n2
        cols.append(xp.sqrt((mx_ - gx) ** 2 + (my_ - gy) ** 2 + mz_ ** 2) / float(refl["vk"][k]))
    for k in range(len(diff["t0"])):
        th = 0.25 * float(diff["t0"][k]) ** 2
        v2 = float(diff["v"][k]) ** 2
        ts = xp.sqrt(th + ((sx - float(diff["x"][k])) ** 2 + (sy - float(diff["y"][k])) ** 2) / v2)
        tg = xp.sqrt(th + ((gx - float(diff["x"][k])) ** 2 + (gy - float(diff["y"][k])) ** 2) / v2)
        cols.append(ts + tg)
    return cols


def synthesize_numpy(m: Patch3DModel) -> np.ndarray:
    s = m.survey
    ns, dt = s.ns, float(s.params["dt"])
    n = m.coords.shape[0]
    out = np.zeros((n, ns), np.float64)
    amps = list(m.refl["amp"]) + list(m.diff["amp"])
    for e, te in enumerate(_event_times(np, m.coords, m.refl, m.diff)):
        _add_events(out, te[:, None], np.full((n, 1), float(amps[e])), dt, m.freq, m.half_width)
    return segy.ibm_roundtrip(out.astype(np.float32))


def synthesize_torch(m: Patch3DModel, device="cuda", chunk: int = 250_000):
    """Same events as synthesize_numpy, computed on a GPU with torch (no IBM
    round trip); returns a float32 tensor [ntr, ns] on ``device``."""
    import torch
    s = m.survey
    ns, dt = s.ns, float(s.params["dt"])
    n = m.coords.shape[0]
    out = torch.zeros((n, ns), dtype=torch.float32, device=device)
    amps = list(m.refl["amp"]) + list(m.diff["amp"])
    k = torch.arange(-m.half_width, m.half_width + 1, device=device, dtype=torch.int64)
    for c0 in range(0, n, chunk):
        c1 = min(n, c0 + chunk)
        c = torch.from_numpy(m.coords[c0:c1]).to(device)
        rows = torch.arange(c1 - c0, device=device, dtype=torch.int64)[:, None] * ns
        flat = out[c0:c1].view(-1)
        for e, te in enumerate(_event_times(torch, c, m.refl, m.diff)):
            idx = torch.floor(te / dt).to(torch.int64)[:, None] + k[None, :]
            ok = (idx >= 0) & (idx < ns)
            a = (math.pi * m.freq * (idx.to(torch.float64) * dt - te[:, None])) ** 2
            w = ((1.0 - 2.0 * a) * torch.exp(-a) * float(amps[e])).to(torch.float32)
            flat.index_add_(0, (rows + idx)[ok], w[ok])
    return out


def patch3d(ntr: int, **kw) -> Survey:
    """A 3-D patch survey with numpy-synthesised samples (see patch3d_model)."""
    m = patch3d_model(ntr, **kw)
    s = m.survey
    s.samples = synthesize_numpy(m)
    return s


def reflectivity_model(nx: int = 200, ny: int = 200, ns: int = 751, dt: float = 0.004, bin_m: float = 25.0,
                       n_refl: int = 12, n_scat: int = 100, seed: int = 5,
                       v_law=(1600.0, 500.0, 100.0, 8000.0), x0: float = 0.0) -> np.ndarray:
    """Reflectivity model of the least-squares workload on the image grid,
    float32 [nx, ny, 1, ns] (stack layout): ``n_refl`` planar dipping
    reflectors and ``n_scat`` point scatterers, seeded.

    A reflector has a centre time t0c ~ U(0.3, 0.85 T) (T the record
    length), a dip theta ~ U(0, 30 deg) along an azimuth ~ U(0, 2 pi) and an
    amplitude ~ +-U(0.5, 1); in every column it is one spike at the
    zero-offset time t0c + 2 tan(theta)/v (lateral distance from the model
    centre), v = v_rms at t0c, split linearly between the two samples around
    it.  A scatterer is a spike of amplitude +-U(0.5, 1) at a random column
    and time ~ U(0.3, 0.9 T).  ``x0`` is the coordinate of column 0 (for
    the lateral velocity term)."""
    rng = np.random.default_rng(seed)
    T = (ns - 1) * dt
    v0, vt, va, lam = v_law
    m = np.zeros((nx, ny, 1, ns), np.float64)
    X, Y = np.meshgrid(np.arange(nx) * bin_m, np.arange(ny) * bin_m, indexing="ij")
    xc, yc = 0.5 * (nx - 1) * bin_m, 0.5 * (ny - 1) * bin_m
    t0c = rng.uniform(0.3, 0.85 * T, n_refl)
    dip = np.radians(rng.uniform(0.0, 30.0, n_refl))
    az = rng.uniform(0.0, 2.0 * math.pi, n_refl)
    amp = rng.uniform(0.5, 1.0, n_refl) * rng.choice([-1.0, 1.0], n_refl)
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    for k in range(n_refl):
        v = v0 + vt * t0c[k] + va * math.sin(2.0 * math.pi * (x0 + xc) / lam)
        p = 2.0 * math.tan(dip[k]) / v
        t0 = t0c[k] + p * (math.cos(az[k]) * (X - xc) + math.sin(az[k]) * (Y - yc))
        tau = t0 / dt
        ok = (tau >= 1.0) & (tau < ns - 2)
        n0 = np.floor(tau[ok]).astype(np.int64)
        f = tau[ok] - n0
        np.add.at(m, (ix[ok], iy[ok], 0, n0), amp[k] * (1.0 - f))
        np.add.at(m, (ix[ok], iy[ok], 0, n0 + 1), amp[k] * f)
    sx = rng.integers(0, nx, n_scat)
    sy = rng.integers(0, ny, n_scat)
    st = np.rint(rng.uniform(0.3, 0.9 * T, n_scat) / dt).astype(np.int64)
    sa = rng.uniform(0.5, 1.0, n_scat) * rng.choice([-1.0, 1.0], n_scat)
    np.add.at(m, (sx, sy, 0, st), sa)
    return m.astype(np.float32)


def lsm_survey_model(ntr: int = 250_000, nx: int = 200, ny: int = 200, ns: int = 751, dt: float = 0.004,
                     seed: int = 5, **kw) -> Patch3DModel:
    """Acquisition of the least-squares workload: ``ntr`` traces with
    midpoints uniform over the nx x ny model at 25 m, offsets U(0, 3000 m),
    random azimuths, ns samples at ``dt``; aperture 3000 m, full physics,
    stack output.  Its data are d = L m (+ noise), not the events of
    patch3d_model."""
    base = dict(ns=ns, dt=dt, nx=nx, ny=ny, bin_m=25.0, max_offset=3000.0, n_refl=0, n_diff=0, freq=25.0,
                aperture=3000.0, seed=seed, mode=1, output=1, name="lsm")
    base.update(kw)
    return patch3d_model(ntr, **base)


def offset_bin_counts(nbins: int = 64, mean: float = 15000.0, lo: int = 2000, hi: int = 40000,
                      seed: int = 4) -> np.ndarray:
    """Traces per offset bin of the batched offset-class workload:
    Poisson(mean) clipped to [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.clip(rng.poisson(mean, nbins), lo, hi).astype(np.int64)


def offset_bins_model(counts, max_offset: float = 4000.0, ns: int = 1001, dt: float = 0.004,
                      nx: int = 160, ny: int = 160, bin_m: float = 12.5, aperture: float = 1500.0,
                      seed: int = 4, **kw) -> Patch3DModel:
    """Batched offset-class survey: len(counts) offset bins of equal width
    over [0, max_offset), bin b holding counts[b] traces with offsets uniform
    inside it (random azimuths, midpoints uniform over the nx x ny patch),
    imaged as offset gathers with one class per bin.  Traces are shuffled so
    that every block mixes all bins."""
    counts = np.asarray(counts, np.int64)
    nb = len(counts)
    dh = max_offset / nb
    rng = np.random.default_rng(seed + 1000)
    off = np.concatenate([rng.uniform(b * dh, (b + 1) * dh, int(n)) for b, n in enumerate(counts)])
    off = off[rng.permutation(off.size)]
    base = dict(ns=ns, dt=dt, nx=nx, ny=ny, bin_m=bin_m, max_offset=max_offset, aperture=aperture,
                seed=seed, output=0, nh=nb, oh=0.0, dh=dh, offsets=off, name="offset_bins")
    base.update(kw)
    return patch3d_model(int(off.size), **base)
