"""Output file assembly without a GPU: the SEG-Y front headers
(write_segy_ebdic_header, Kirchhoff.c:729-814) and the combine step
(combine_all_files, :821-874), against the compiled reference's own files
when the reference is present."""
from __future__ import annotations

import tempfile
from pathlib import Path

import numpy as np
import pytest

from oracle.refbuild import REFERENCE_SOURCE
from random_gb300 import synth
from random_gb300.migration import combine_su, segy_front_headers


def _u16(b, off):
    return int.from_bytes(b[off:off + 2], "big")


def test_front_header_fields(kpstm_lib):
    s = synth.line2d(n_cmp=10, n_off=4, ns=301, seed=3)
    h = segy_front_headers(s.params)
    assert len(h) == 3600
    assert h[:23] == b"written by G. O'Brien\n\x00"
    b = h[3200:]
    assert _u16(b, 16) == 4000 and _u16(b, 20) == 301 and _u16(b, 22) == 301
    assert _u16(b, 24) == 5 and _u16(b, 26) == 1 and _u16(b, 28) == 1 and _u16(b, 30) == 1
    assert _u16(b, 12) == (10 * 1 * 4) & 0xFFFF


@pytest.mark.skipif(not REFERENCE_SOURCE.exists(), reason="reference checkout absent")
def test_front_headers_and_combine_match_the_reference(kpstm_lib):
    from oracle import refbuild
    s = synth.line2d(n_cmp=12, n_off=4, ns=201, seed=5, aperture_m=300.0)
    jobs = 3
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        s.write_files(td / "d.segy", td / "v.segy")
        b = refbuild.compile(refbuild.RefConfig(**s.ref_config(jobs_x=jobs, jobs_y=1)), tag="hdr")
        refbuild.run(b, td / "run", td / "d.segy", td / "v.segy", nprocs=jobs)
        img = td / "run" / "image_dir"
        text = (img / "ebdic_header.bin").read_bytes()
        binh = (img / "binary_header.bin").read_bytes()
        mine = segy_front_headers(dict(s.params, jobs_x=jobs, jobs_y=1, job_id=0))
        # the reference leaves text bytes 44.. and binary bytes 12-13 uninitialised
        assert mine[:44] == text[:44]
        assert mine[3200:3212] == binh[:12] and mine[3214:] == binh[14:]
        slabs = [img / f"image{j}.su" for j in range(jobs)]
        combine_su(td / "out.segy", dict(s.params, jobs_x=jobs, jobs_y=1, job_id=0), slabs)
        out = (td / "out.segy").read_bytes()
        want = b"".join(p.read_bytes() for p in slabs)   # the script's cat of image0..imageN
        assert out[3600:] == want and len(out) == 3600 + len(want)
        # the script itself lists the slabs in job order after the two headers
        script = (img / "combine_script").read_text().split("\n")
        assert script[0].startswith("cat ebdic_header.bin binary_header.bin")
        assert [ln.split()[1] for ln in script[1:1 + jobs]] == [f"image{j}.su" for j in range(jobs)]


def test_velocity_loader_reads_the_written_model(kpstm_lib, tmp_path):
    """The velocity file the harness writes for the reference, read back
    with build_vel_model's binning, equals the grid it was written from."""
    from random_gb300.migration import velocity_from_segy
    s = synth.patch3d(ntr=20, ns=151, dt=0.004, nx=6, ny=4, bin_m=25.0, max_offset=600.0, n_refl=1, n_diff=1,
                      aperture=200.0, seed=4)
    s.write_files(tmp_path / "d.segy", tmp_path / "v.segy")
    v = s.velocity
    got, nsm, dtm = velocity_from_segy((tmp_path / "v.segy").read_bytes(), v.n_iline, v.n_xline, v.o_iline,
                                       v.o_xline, v.d_iline, v.d_xline)
    assert nsm == v.nsm and dtm == np.float32(v.dtm)
    assert np.array_equal(got.view(np.uint32), np.asarray(v.vrms, np.float32).reshape(got.shape).view(np.uint32))
    # a grid larger than the file: the extra cells stay 0; a shifted origin drops rows
    got2, _, _ = velocity_from_segy((tmp_path / "v.segy").read_bytes(), v.n_iline + 2, v.n_xline, v.o_iline,
                                    v.o_xline, v.d_iline, v.d_xline)
    assert np.array_equal(got2[:v.n_iline], got) and not got2[v.n_iline:].any()
    got3, _, _ = velocity_from_segy((tmp_path / "v.segy").read_bytes(), v.n_iline, v.n_xline, v.o_iline + 2,
                                    v.o_xline, v.d_iline, v.d_xline)
    assert np.array_equal(got3[:v.n_iline - 2], got[2:]) and not got3[v.n_iline - 2:].any()
