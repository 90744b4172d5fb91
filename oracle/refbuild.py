"""Build and run the reference ``Kirchhoff.c`` as the CPU oracle / CPU baseline.

Test infrastructure only.  The product never imports this module; only
``tests/``, ``__graft_entry__`` (build + smoke check) and ``bench.py``'s CPU
baseline leg use it.

The reference keeps its whole configuration in ``#define`` lines
(Kirchhoff.c:17-65) that cannot be overridden with ``-D``.  ``patch()``
rewrites each of those lines so that the value comes from a ``KREF_<name>``
macro supplied on the compiler command line, and points the hard-coded file
paths (Kirchhoff.c:21, 30-31, 62) at fixed names relative to the working
directory.  Nothing else in the source is touched.  The patched copy lives in
``oracle/_ref/`` (git-ignored, but shipped with the tree), so that a machine
without the reference checkout can still compile it for any configuration.

MPI and FFTW3 are absent here; ``oracle/shim`` supplies a single-communicator
MPI stand-in (rank/size from the environment) and an FFTW3-compatible DFT.

Build line: the reference documents
``mpicc -o KTM Kirchhoff_time.c -lm -lfftw3 -w -ffast-math`` (Kirchhoff.c:3),
i.e. no optimisation level.  ``compile(..., opt="-O0")`` reproduces it and is
what parity is pinned against; the CPU baseline timing uses ``-O3
-ffast-math`` (a faster reference, so a more conservative speed-up).
"""
from __future__ import annotations

import hashlib
import os
import re
import shutil
import subprocess
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
SHIM_DIR = HERE / "shim"
PATCHED = REF_DIR / "Kirchhoff_kref.c"
# the reference checkout: KPSTM_REFERENCE_DIR, else a "reference" directory
# beside this repository
REFERENCE_SOURCE = Path(os.environ.get("KPSTM_REFERENCE_DIR", HERE.parent.parent / "reference")) / "Kirchhoff.c"

# Numeric configuration macros of Kirchhoff.c:17-65, in file order.
NUMERIC = [
    "run_test", "NVel_ilines", "NVel_xlines", "dVel_ilines", "dVel_xlines",
    "oVel_ilines", "oVel_xlines", "Startiline", "Endiline", "Startxline",
    "Endxline", "INCiline", "INCxline", "dh", "nh", "oh", "ox", "oy",
    "angleEtoN", "iline_distance", "xline_distance", "aperture",
    "anti_alias_cutoff", "ntblock", "number_mpi_jobsX", "number_mpi_jobsY",
]
# String macros and the fixed relative names they are pointed at.
STRINGS = {
    "input_vel": "vel.segy",
    "input_data": "data.segy",
    "output_data": "pstm_gathers.sgy",
    "image_dir": "image_dir",
}
# Macros that the reference uses in integer arithmetic (integer division in
# Kirchhoff.c:539, 1357-1358, loop bounds); they must be passed as integers.
INTEGER = {"run_test", "NVel_ilines", "NVel_xlines", "dVel_ilines", "dVel_xlines",
           "oVel_ilines", "oVel_xlines", "Startiline", "Endiline", "Startxline",
           "Endxline", "nh", "ntblock", "number_mpi_jobsX", "number_mpi_jobsY"}


def patch(source: Path = REFERENCE_SOURCE, dest: Path = PATCHED) -> Path:
    """Write the patched copy of the reference into ``oracle/_ref``."""
    text = source.read_text(encoding="latin-1")
    lines = text.split("\n")
    found = set()
    for i, line in enumerate(lines[:80]):
        m = re.match(r"^#define\s+(\w+)\s+(.*)$", line)
        if not m:
            continue
        name = m.group(1)
        if name in STRINGS:
            lines[i] = f'#define {name} "{STRINGS[name]}"'
            found.add(name)
        elif name in NUMERIC:
            lines[i] = f"#define {name} (KREF_{name})"
            found.add(name)
    missing = (set(NUMERIC) | set(STRINGS)) - found
    if missing:
        raise RuntimeError(f"reference define block changed; not found: {sorted(missing)}")
    dest.parent.mkdir(parents=True, exist_ok=True)
    dest.write_text("\n".join(lines), encoding="latin-1")
    return dest


def have_patched() -> bool:
    return PATCHED.exists()


def ensure_patched() -> Path:
    if REFERENCE_SOURCE.exists():
        if not PATCHED.exists() or PATCHED.stat().st_mtime < REFERENCE_SOURCE.stat().st_mtime:
            patch()
    if not PATCHED.exists():
        raise FileNotFoundError("patched reference source missing and reference checkout absent")
    return PATCHED


def _fmt(name: str, v) -> str:
    if name in INTEGER:
        if int(v) != v:
            raise ValueError(f"{name} must be an integer, got {v}")
        return str(int(v))
    return repr(float(v))


@dataclass
class RefConfig:
    """Values for the reference's compile-time configuration (Kirchhoff.c:17-65)."""
    NVel_ilines: int
    NVel_xlines: int
    dVel_ilines: int
    dVel_xlines: int
    oVel_ilines: int
    oVel_xlines: int
    Startiline: int
    Endiline: int
    Startxline: int
    Endxline: int
    INCiline: float
    INCxline: float
    dh: float
    nh: int
    oh: float
    ox: float
    oy: float
    angleEtoN: float
    iline_distance: float
    xline_distance: float
    aperture: float
    anti_alias_cutoff: float
    ntblock: int = 50000
    number_mpi_jobsX: int = 1
    number_mpi_jobsY: int = 1
    run_test: int = 1

    def defines(self) -> list[str]:
        return [f"-DKREF_{k}={_fmt(k, getattr(self, k))}" for k in NUMERIC]


def compile(cfg: RefConfig, opt: str = "-O0", fast_math: bool = True, tag: str | None = None) -> Path:
    """Compile the patched reference for ``cfg``; returns the binary path."""
    src = ensure_patched()
    flags = [opt, "-w"] + (["-ffast-math"] if fast_math else []) + cfg.defines()
    key = hashlib.sha1((" ".join(flags) + src.read_text(encoding="latin-1")).encode()).hexdigest()[:12]
    out = REF_DIR / f"ktm_{tag or 'cfg'}_{key}"
    if out.exists():
        return out
    # The FFTW stand-in is a separately built library, as FFTW is: it gets
    # its own flags, not the reference's -ffast-math.
    shim_obj = REF_DIR / f"fftw_shim_{key}.o"
    subprocess.run(["gcc", "-std=gnu17", "-O2", "-ffp-contract=off", "-c", f"-I{SHIM_DIR}",
                    str(SHIM_DIR / "fftw_shim.c"), "-o", str(shim_obj)], check=True, capture_output=True)
    cmd = ["gcc", "-std=gnu17", *flags, f"-I{SHIM_DIR}", str(src), str(shim_obj), "-lm", "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True)
    shim_obj.unlink()
    return out


@dataclass
class RefRun:
    workdir: Path
    seconds: float
    jobs: int
    stdout: list[str] = field(default_factory=list)


def run(binary: Path, workdir: Path, data_segy: Path, vel_segy: Path, nprocs: int = 1,
        timeout: float = 3600.0) -> RefRun:
    """Run the reference with ``nprocs`` independent ranks in ``workdir``.

    Each rank runs the jobs ``job = rank, rank + nprocs, ...`` of the
    reference's own loop (Kirchhoff.c:347).  Rank 0's header/QC files and the
    output directory are created by the reference itself; the directory is
    created here first because the ranks do not synchronise.
    """
    workdir.mkdir(parents=True, exist_ok=True)
    for name, src in (("data.segy", data_segy), ("vel.segy", vel_segy)):
        dst = workdir / name
        if dst.exists() or dst.is_symlink():
            dst.unlink()
        os.symlink(os.path.abspath(src), dst)
    (workdir / "image_dir").mkdir(exist_ok=True)
    env = dict(os.environ)
    procs = []
    t0 = time.perf_counter()
    for r in range(nprocs):
        env_r = dict(env, KPSTM_REF_RANK=str(r), KPSTM_REF_SIZE=str(nprocs))
        procs.append(subprocess.Popen([str(binary)], cwd=workdir, env=env_r,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                      stdin=subprocess.DEVNULL))
    outs = []
    for p in procs:
        out, _ = p.communicate(timeout=timeout)
        outs.append(out.decode(errors="replace"))
        if p.returncode not in (0, None):
            # The reference's main() has no return statement; its exit status
            # is whatever MPI_Finalize's stand-in returned last (0).
            raise RuntimeError(f"reference rank exited {p.returncode}:\n{outs[-1][-2000:]}")
    dt = time.perf_counter() - t0
    return RefRun(workdir=workdir, seconds=dt, jobs=nprocs, stdout=outs)


def read_su(path: Path, ns: int) -> tuple[np.ndarray, np.ndarray]:
    """Parse a big-endian SU file written by Kirchhoff.c:1482-1593.

    Returns (headers [ntr, 60] as big-endian-decoded int32 words, data [ntr, ns]
    float32).  Header words that hold 16-bit fields are returned raw.
    """
    raw = np.fromfile(path, dtype=np.uint8)
    rec = 240 + 4 * ns
    if raw.size % rec:
        raise ValueError(f"{path}: size {raw.size} is not a multiple of {rec}")
    ntr = raw.size // rec
    raw = raw.reshape(ntr, rec)
    hdr = raw[:, :240].copy().view(">i4").astype(np.int32)
    data = raw[:, 240:].copy().view(">f4").astype(np.float32)
    return hdr, data


def read_image(workdir: Path, ns: int, n_jobs: int) -> tuple[np.ndarray, np.ndarray]:
    """Concatenate image<job>.su in job order, as the reference's combine
    script does (Kirchhoff.c:852-872)."""
    hs, ds = [], []
    for j in range(n_jobs):
        h, d = read_su(workdir / "image_dir" / f"image{j}.su", ns)
        hs.append(h)
        ds.append(d)
    return np.concatenate(hs), np.concatenate(ds)


def clean(workdir: Path) -> None:
    shutil.rmtree(workdir, ignore_errors=True)
