"""Generate the golden fixtures in this directory from the reference itself.

Each fixture is a small seeded survey imaged by the reference's own
``kirchhoff()`` (Kirchhoff.c), compiled from the reference checkout with the
documented flags by ``oracle/refbuild.py`` and run as independent ranks.
Stored per fixture (``<name>.npz``):

    params        JSON of the kpstm_params values
    vel_*         the v_rms grid (kpstm_velocity fields) and values
    headers       [ntr, 60] int32 trace-header words (host order)
    ibm           [ntr, ns] uint32 IBM sample words (the exact file contents)
    image         [nx_total, ny, nh, ns] float32: the SU files of all jobs,
                  concatenated in job order (the reference's combine script)
    su_headers    [ntraces, 60] int32: the SU header words it wrote
    jobs          (jobs_x, jobs_y)

Also ``line2d_full.json``: the reference's image of the full 2-D
line (synth.line2d(): 200 CMPs x 48 offsets, 1001 samples, 1.61e9 pairs,
one rank), too large to store, recorded as the SHA-256 of its float32
bytes ([traces][ns], little-endian, SU trace order) with its norm.

Run here (needs the reference checkout and gcc):
    python tests/golden/make_golden.py [name ...]
"""
from __future__ import annotations

import hashlib
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import refbuild  # noqa: E402
from random_gb300 import segy, synth  # noqa: E402

HERE = Path(__file__).resolve().parent


def _line_overhang_coarse_velocity():
    """2-D line of 10 CMPs cut into 3 slabs of ceil(10/3) = 4 inlines, so that
    the last slab runs 2 inlines past the end (Kirchhoff.c:266-300), with a
    v_rms grid that covers them, varies along the line and is sampled at
    twice the trace interval (the velocity sample of t is round(t dt / dtm),
    Kirchhoff.c:1357-1378)."""
    s = synth.line2d(n_cmp=10, n_off=4, ns=201, seed=8, aa_cutoff=40.0)
    u = s.info["units_per_metre"]
    v = s.velocity
    nil, nsm, dtm = 12, 102, 2.0 * v.dtm
    t0 = np.arange(nsm) * dtm
    vt = ((1500.0 + 600.0 * t0[None, :] + 15.0 * np.arange(nil)[:, None]) * u).astype(np.float32)
    s.velocity = synth.Velocity(n_iline=nil, n_xline=1, nsm=nsm, o_iline=v.o_iline, o_xline=v.o_xline,
                                d_iline=1, d_xline=1, dtm=dtm, vrms=segy.ibm_roundtrip(vt[:, None, :].copy()))
    return s


def fixtures():
    """name -> (survey, jobs_x, jobs_y)"""
    return {
        # 2-D line, odd ns (the anti-alias mirror zeroes bins ns/2, ns/2+1),
        # low-pass "off", one job
        "g1_line_oddns": (synth.line2d(n_cmp=16, n_off=6, ns=251, seed=3), 1, 1),
        # 2-D line, even ns, 40 Hz low-pass, image cut into 3 slabs
        "g2_line_slabs": (synth.line2d(n_cmp=12, n_off=6, ns=300, seed=5, aa_cutoff=40.0), 3, 1),
        # 3-D, rotated survey with a non-zero origin, 4 offset classes (some
        # traces beyond the last class), slab cull active, 2 x 2 slabs
        "g3_patch_rotated": (synth.patch3d(ntr=240, ns=161, dt=0.004, nx=8, ny=6, bin_m=25.0,
                                           max_offset=1000.0, n_refl=2, n_diff=6, freq=25.0,
                                           aperture=300.0, aa_cutoff=60.0, seed=7, mode=0,
                                           output=0, nh=4, oh=0.0, dh=200.0, rotate_deg=30.0,
                                           origin=(1000.0, 2000.0)), 2, 2),
        # 2-D line, the last of 3 slabs past the end inline, coarse and
        # laterally varying v_rms
        "g4_line_overhang": (_line_overhang_coarse_velocity(), 3, 1),
        # 3-D, 6 x 5 columns in 2 x 2 slabs: the second xline slab (3 of
        # ceil(5/2)) runs one xline past the end (the v_rms grid is one
        # xline wide, so it covers it); 3 offset classes, 40 Hz low-pass
        "g5_patch_xline_overhang": (synth.patch3d(ntr=200, ns=180, dt=0.004, nx=6, ny=5, bin_m=25.0,
                                                  max_offset=900.0, n_refl=2, n_diff=5, freq=25.0,
                                                  aperture=400.0, aa_cutoff=40.0, seed=9, mode=0,
                                                  output=0, nh=3, oh=0.0, dh=300.0), 2, 2),
    }


def run_reference(s, jx: int, jy: int, work: Path):
    s.write_files(work / "data.segy", work / "vel.segy")
    cfg = refbuild.RefConfig(**s.ref_config(jobs_x=jx, jobs_y=jy))
    binary = refbuild.compile(cfg, tag="golden")
    refbuild.run(binary, work / "run", work / "data.segy", work / "vel.segy", nprocs=jx * jy)
    return refbuild.read_image(work / "run", s.ns, jx * jy)


def line2d_full() -> dict:
    s = synth.line2d()
    with tempfile.TemporaryDirectory() as td:
        _, img = run_reference(s, 1, 1, Path(td))
    img = np.ascontiguousarray(img, dtype="<f4")
    return {"survey": "synth.line2d()", "traces": int(img.shape[0]), "ns": int(img.shape[1]),
            "jobs": [1, 1], "reference": "Kirchhoff.c via oracle/refbuild.py, -O0 -w -ffast-math, one rank",
            "sha256": hashlib.sha256(img.tobytes()).hexdigest(),
            "l2_norm": float(np.linalg.norm(img.astype(np.float64))),
            "max_abs": float(np.max(np.abs(img)))}


def main(names=()):
    """All fixtures, or only the named ones (``line2d_full`` for the JSON)."""
    if not names or "line2d_full" in names:
        (HERE / "line2d_full.json").write_text(json.dumps(line2d_full(), indent=1) + "\n")
        print("line2d_full.json")
    for name, (s, jx, jy) in fixtures().items():
        if names and name not in names:
            continue
        with tempfile.TemporaryDirectory() as td:
            hdr, img = run_reference(s, jx, jy, Path(td))
        v = s.velocity
        np.savez_compressed(
            HERE / f"{name}.npz",
            params=json.dumps(s.params), jobs=np.array([jx, jy]),
            vel_grid=np.array([v.n_iline, v.n_xline, v.nsm, v.o_iline, v.o_xline, v.d_iline, v.d_xline]),
            vel_dtm=np.float32(v.dtm), vel=v.vrms.astype(np.float32),
            headers=s.headers, ibm=segy.ieee_to_ibm(s.samples), image=img.astype(np.float32),
            su_headers=hdr.astype(np.int32))
        print(name, s.ntr, "traces ->", img.shape)


if __name__ == "__main__":
    main(sys.argv[1:])
