"""Build libkpstm.so in-tree: nvcc for the CUDA translation unit (sm_103a
only), gcc for the host C, linked by nvcc with the static CUDA runtime.

    python -m random_gb300.build          # build if sources changed
    python -m random_gb300.build --force

The two translation units compile in parallel.  ``-Xptxas -v`` output
(registers, spills, shared memory per kernel) goes to
``random_gb300/_build/ptxas.log``.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OUT = PKG / "libkpstm.so"
BUILD = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise FileNotFoundError("nvcc not found")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.c")) + sorted(CSRC.glob("*.h")) + \
        sorted(CSRC.glob("*.cuh")) + [INCLUDE / "kpstm.h"]


def stale() -> bool:
    if not OUT.exists():
        return True
    t = OUT.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not stale():
        return OUT
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    cu_obj = BUILD / "kpstm_cuda.o"
    c_obj = BUILD / "kpstm_host.o"
    cu_cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-v", f"-I{INCLUDE}", "-c", str(CSRC / "kpstm_cuda.cu"), "-o", str(cu_obj)]
    c_cmd = ["gcc", "-std=gnu17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", f"-I{INCLUDE}",
             "-c", str(CSRC / "kpstm_host.c"), "-o", str(c_obj)]
    p_cu = subprocess.Popen(cu_cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    p_c = subprocess.Popen(c_cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    out_c, _ = p_c.communicate()
    out_cu, _ = p_cu.communicate()
    (BUILD / "ptxas.log").write_bytes(out_cu)
    if p_c.returncode:
        raise RuntimeError("gcc failed:\n" + out_c.decode(errors="replace"))
    if p_cu.returncode:
        raise RuntimeError("nvcc failed:\n" + out_cu.decode(errors="replace")[-6000:])
    tmp = OUT.with_suffix(f".so.{os.getpid()}")
    link = [nvcc, *ARCH, "-shared", "-cudart", "static", str(cu_obj), str(c_obj), "-o", str(tmp)]
    r = subprocess.run(link, capture_output=True)
    if r.returncode:
        raise RuntimeError("link failed:\n" + (r.stdout + r.stderr).decode(errors="replace"))
    os.replace(tmp, OUT)
    if verbose:
        sys.stdout.write(out_cu.decode(errors="replace"))
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
