"""Load the golden fixtures of tests/golden into synth.Survey objects."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from random_gb300 import segy, synth

GOLDEN = Path(__file__).resolve().parent / "golden"
NAMES = ["g1_line_oddns", "g2_line_slabs", "g3_patch_rotated", "g4_line_overhang", "g5_patch_xline_overhang"]


def load(name: str):
    z = np.load(GOLDEN / f"{name}.npz")
    params = json.loads(str(z["params"]))
    g = [int(x) for x in z["vel_grid"]]
    vel = synth.Velocity(n_iline=g[0], n_xline=g[1], nsm=g[2], o_iline=g[3], o_xline=g[4],
                         d_iline=g[5], d_xline=g[6], dtm=float(z["vel_dtm"]), vrms=z["vel"])
    samples = segy.ibm_to_ieee(z["ibm"])
    s = synth.Survey(name, params, vel, z["headers"], samples)
    jx, jy = (int(v) for v in z["jobs"])
    return s, jx, jy, z["image"], z["su_headers"], z["ibm"]


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def line2d_golden() -> dict:
    """The compiled reference's full 2-D line image as recorded by
    tests/golden/make_golden.py (SHA-256 of its float32 bytes and norms)."""
    return json.loads((GOLDEN / "line2d_full.json").read_text())


def image_sha256(img) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(img, dtype="<f4").tobytes()).hexdigest()
