#!/usr/bin/env python
"""Benchmark: 3-D Kirchhoff PSTM, 1e6 traces x 1501 samples (2 ms) into a
400 x 400 x 1501 stack image at 25 m bins, aperture 3000 m, triangle
anti-alias, spreading + obliquity weights (KPSTM_MODE_FULL), fp32.

A step is one block of 50,000 traces (the reference's ntblock,
Kirchhoff.c:63) migrated into the whole image: kpstm_add_traces_device on
inputs already in HBM (the survey is synthesised on the GPU once, 6 GB).
Metric: Gsample-trace pairs/s, one pair = one (trace, in-aperture image
column, output sample) = one pass of Kirchhoff.c:1374-1399.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun each rank images its own slab of a wider survey (the
reference's independent image slabs, Kirchhoff.c:280-300), so per-GPU work
is fixed ("weak" scaling) and there is no data-path collective.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gsample-trace pairs/s"
UNIT = "Gpairs/s"
NS, DT = 1501, 0.002
NX = NY = 400
SURVEY_TRACES = 1_000_000
STEP_TRACES = 50_000
PEAKS = {"hbm_gbs": 6800.0, "source": "fallback"}


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "sm_max_mhz": float(d.get("sm_max_mhz", 2070.0)),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0, "source": "fallback"}


# --------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        if shutil.which("nvidia-smi") is None:
            return
        self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                   "--format=csv,noheader,nounits", "-lms", "200"],
                                  stdout=self.f, stderr=subprocess.DEVNULL)

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            c = [x.strip() for x in line.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                smax.append(float(c[2]))
            except ValueError:
                continue
            for n, v in zip(names, c[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------- workload
def survey_model(rank: int = 0, ntr: int = SURVEY_TRACES):
    from random_gb300 import multirank, synth
    # each rank: its own 10 km x 10 km slab (x shifted), same statistics
    return synth.patch3d_model(ntr, ns=NS, dt=DT, nx=NX, ny=NY, bin_m=25.0, max_offset=4000.0,
                               n_refl=8, n_diff=200, freq=30.0, aperture=3000.0, aa_cutoff=100.0,
                               seed=2 + rank, mode=1, output=1,
                               x_shift=multirank.weak_scaling_shift(rank, 20000.0))


def algorithmic_bytes_per_step(model, ntr_step: int, row_floats: int) -> int:
    """Compulsory bytes of one imaging launch: the block's tap tables read
    once, geometry, the image accumulators (sums + counts) read and written
    once, and the velocity rows."""
    ncol = NX * NY
    return ntr_step * row_floats * 4 + ntr_step * 32 + ncol * NS * 4 * 2 * 2 + NX * NS * 8


# ------------------------------------------------------------ CPU baseline
def cpu_sample(n_traces: int, n_procs: int, opt: str = "-O3"):
    """The reference's kirchhoff() on this host's cores: the image is cut
    into 400 one-iline slabs (its own decomposition, Kirchhoff.c:280-300) and
    n_procs of them, spread across the image, run as independent ranks over
    the first n_traces traces of the same survey.  Returns (pairs, seconds)."""
    from oracle import refbuild
    from random_gb300 import synth
    sm = synth.patch3d_model(SURVEY_TRACES, ns=NS, dt=DT, nx=NX, ny=NY, bin_m=25.0, max_offset=4000.0,
                             n_refl=8, n_diff=200, freq=30.0, aperture=3000.0, aa_cutoff=100.0, seed=2,
                             mode=1, output=1, trace_slice=slice(0, n_traces))
    s = sm.survey
    s.samples = synth.synthesize_numpy(sm)
    jobs = sorted({int((k + 0.5) * NX / n_procs) for k in range(n_procs)})
    work = Path(tempfile.mkdtemp(prefix="kref_"))
    try:
        s.write_files(work / "data.segy", work / "vel.segy")
        cfg = refbuild.RefConfig(**s.ref_config(jobs_x=NX, jobs_y=1, ntblock=s.ntr))
        binary = refbuild.compile(cfg, opt=opt, tag="bench")
        (work / "run" / "image_dir").mkdir(parents=True, exist_ok=True)
        for name in ("data.segy", "vel.segy"):
            os.symlink(work / name, work / "run" / name)
        t0 = time.perf_counter()
        procs = [subprocess.Popen([str(binary)], cwd=work / "run", stdout=subprocess.DEVNULL,
                                  stderr=subprocess.DEVNULL, stdin=subprocess.DEVNULL,
                                  env=dict(os.environ, KPSTM_REF_RANK=str(j), KPSTM_REF_SIZE=str(NX)))
                 for j in jobs]
        for p in procs:
            p.wait()
        secs = time.perf_counter() - t0
        if any(p.returncode for p in procs):
            raise RuntimeError("reference rank failed")
    finally:
        shutil.rmtree(work, ignore_errors=True)
    # pairs: in-aperture (trace, column) of the sampled slabs, float32 test as Kirchhoff.c:1351-1354
    p = s.params
    h = s.headers.astype(np.float64)
    cx = (0.5 * (h[:, 18] + h[:, 20])).astype(np.float32)
    cy = (0.5 * (h[:, 19] + h[:, 21])).astype(np.float32)
    IY = ((p["start_xline"] + np.arange(NY)) * 25.0).astype(np.float32)
    pairs = 0
    for j in jobs:
        IX = np.float32((p["start_iline"] + j) * 25.0)
        dx = IX - cx
        dy = IY[None, :] - cy[:, None]
        d = np.sqrt(dx[:, None] * dx[:, None] + dy * dy)
        pairs += int((d < np.float32(3000.0)).sum()) * NS
    return pairs, secs, len(jobs)


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ----------------------------------------------------------------- our arm
def run_ours(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    from random_gb300 import build, capi, multirank, segy, synth
    from random_gb300.migration import Migration

    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    peaks = load_peaks()
    model = survey_model(rank, args.survey_traces)
    s = model.survey
    ntr = s.ntr
    hdr_be = np.ascontiguousarray(segy.headers_be(s.headers))
    d_hdr = torch.from_numpy(hdr_be).to(dev)
    d_smp = synth.synthesize_torch(model, device=dev)
    torch.cuda.synchronize()
    block = args.traces_per_step
    nblocks = ntr // block
    row_bytes = NS * 4

    prm = dict(s.params, precision=1 if args.precision == "bf16" else 0)
    m = Migration(prm, s.velocity)
    # a dedicated (non-default) stream shared by the library and the timers
    stream = torch.cuda.Stream(device=dev)
    m.set_stream(stream.cuda_stream)

    tuned = None
    if args.autotune > 0:
        cfg, tune_ms = m.autotune(d_hdr.data_ptr(), d_smp.data_ptr(), args.autotune)
        tuned = dict(cfg, sample_traces=args.autotune, block_ms=round(tune_ms, 3))

    def step(i):
        b = i % nblocks
        m.add_traces_device(d_hdr.data_ptr() + b * block * 240, d_smp.data_ptr() + b * block * row_bytes, block)

    for i in range(args.warmup):
        step(i)
    m.synchronize()
    m.profile(True)
    m.profile_read()
    pairs0 = m.pairs()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(args.steps):
        step(args.warmup + i)
    e1.record(stream)
    torch.cuda.synchronize()
    m.synchronize()
    clk = clocks.stop()
    if world > 1:
        dist.barrier()
    elapsed = e0.elapsed_time(e1) / 1e3
    prof = m.profile_read()
    m.profile(False)
    launch_cfg = m.launch_config()
    pairs = m.pairs() - pairs0
    elapsed_max, pairs_all = multirank.reduce_timing(elapsed, float(pairs), device=dev)
    value = pairs_all / elapsed_max / 1e9

    # roofline of the imaging kernel (dominant: see profile shares)
    launches = max(1, int(prof["image_launches"]))
    t_launch = prof["image_ms"] / 1e3 / launches
    row_floats = 2 * (NS + 2 * m.dims["trange_max"] - 2)
    row_floats = 8 + ((row_floats + 3) & ~3)  # geometry header + taps
    b_alg = algorithmic_bytes_per_step(model, block, row_floats)
    achieved = b_alg / t_launch / 1e9
    pairs_per_launch = pairs / launches
    # DRAM traffic per launch from ncu (dram__bytes_read + write) of a
    # 5,000-trace launch of the default kernel (3 CTAs/SM, K = 16, persistent)
    # into the same image: 3.944e9 bytes, of which the tap tables are 5,000
    # rows; the accumulator part is fixed, the table part grows with the traces
    traffic = 3.944e9 + (block - 5000) * row_floats * 4
    # issue-slot roofline: warp instructions per pair from a capture of the same
    # launch (37.2 per 32 pairs) against 4 schedulers x SMs x the SM clock
    instr_per_pair = 37.23 / 32
    issue_peak = 4 * 152 * (clk.get("sm_mhz") or peaks["sm_max_mhz"]) * 1e6
    issue_achieved = pairs_per_launch / t_launch * instr_per_pair
    roofline = {
        "bound": "hbm", "achieved": round(achieved, 3), "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": round(achieved / peaks["hbm_gbs"], 6), "traffic": round(traffic),
        "traffic_source": "ncu dram bytes of a 5,000-trace launch, table part scaled to the block",
        "peak_source": peaks["source"], "kernel": "k_image (full mode)",
        "algorithmic_bytes_per_launch": b_alg, "launch_ms": round(t_launch * 1e3, 3),
        "pairs_per_launch": pairs_per_launch,
        "binding": "SM instruction issue and latency (no tensor work; HBM bytes per pair are ~1e-3; "
                   "FMA, ALU and SFU pipes each at most ~55% busy): see profiles/",
        "issue": {"achieved": round(issue_achieved / 1e12, 4), "peak": round(issue_peak / 1e12, 4),
                  "unit": "T warp-instr/s", "frac": round(issue_achieved / issue_peak, 4),
                  "instr_per_pair_source": "ncu smsp__inst_executed / pairs, 5,000-trace launch"},
        "image_kernel_share": round(prof["image_ms"] / (prof["image_ms"] + prof["prep_ms"]), 4),
    }
    del m

    # -------- e2e through the C ABI from pinned host memory
    e2e = None
    if not args.no_e2e:
        nb = min(nblocks, 4)
        h_hdr = torch.from_numpy(hdr_be[:nb * block]).pin_memory()
        h_smp = d_smp[:nb * block].cpu().pin_memory()
        m2 = Migration(prm, s.velocity)
        m2.set_launch(**launch_cfg)
        out = torch.empty((NX, NY, 1, NS), dtype=torch.float32).pin_memory()
        # one untimed block to create the staging buffers
        m2.add_traces_ptr(h_hdr.data_ptr(), h_smp.data_ptr(), block)
        m2.synchronize()
        m2.reset()
        pe0 = m2.pairs()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(args.steps):
            b = i % nb
            m2.add_traces_ptr(h_hdr.data_ptr() + b * block * 240, h_smp.data_ptr() + b * block * row_bytes, block)
        m2.finish_ptr(out.data_ptr())
        t_e2e = time.perf_counter() - t0
        pe = m2.pairs() - pe0
        del m2
        e2e = {"value": round(pe / t_e2e / 1e9, 4), "unit": UNIT,
               "h2d_bytes_per_step": block * (240 + row_bytes),
               "d2h_bytes_per_step": int(out.numel() * 4 / args.steps) + 4,
               "note": "kpstm_add_traces from pinned host buffers every step; one kpstm_finish "
                       "(image to host) closes the timed region; wall clock"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cores = host_cores()
        pairs_c, secs_c, nslab = cpu_sample(args.cpu_traces, cores)
        cpu = {"value": round(pairs_c / secs_c / 1e9, 4), "unit": UNIT, "cores": nslab, "kind": "reference",
               "sample": f"reference kirchhoff() (-O3 -ffast-math, MPI/FFTW stand-ins) on {nslab} of its "
                         f"400 one-iline slabs, first {args.cpu_traces} traces of the survey, one rank per "
                         f"core: {pairs_c} pairs in {secs_c:.2f} s"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(elapsed_max / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "fp32" else "bf16 store, f32 compute (Kahan)",
            "data": "synthetic (seeded 3-D survey: 8 dipping reflectors + 200 diffractors, 30 Hz Ricker)",
            "config": {"workload": "3-D PSTM, 1e6 traces x 1501 samples @ 2 ms, 400x400x1501 stack image at "
                                   "25 m, aperture 3000 m, triangle anti-alias + spreading/obliquity, fp32",
                       "traces_per_step": block, "survey_traces": ntr, "mode": "full",
                       "l2": "inputs larger than L2: 613 MB tap tables + 1.9 GB image accumulators per step",
                       "parallelism": f"image slabs x{world}", "launch": launch_cfg, "autotuned": tuned},
            "gpu_launches": int(prof["image_launches"] + prof["other_launches"]),
            "pairs": int(pairs_all), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "profile_ms": {"image": round(prof["image_ms"], 3), "prep": round(prof["prep_ms"], 3)},
        }
        print(json.dumps(line), flush=True)


# ------------------------------------------------- further workloads (not the bench line)
def _timed_steps(step, warmup, steps, stream, after_warmup=None):
    import torch
    for i in range(warmup):
        step(i)
    torch.cuda.synchronize()
    if after_warmup:
        after_warmup()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        step(warmup + i)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3, clocks.stop()


def run_offset_bins(args):
    """64 offset bins over 0-4000 m, Poisson(15000) traces per bin clipped to
    [2000, 40000] (960,790 traces), ns = 1001 at 4 ms, each bin imaged into
    160 x 160 x 1001 offset gathers, reference operator with BF16 trace
    storage and Kahan accumulation; the launch configuration is autotuned on
    the first 8,000 traces, then each block is imaged by one persistent launch
    replayed from a CUDA graph.  A step is a block of traces of all bins."""
    import torch
    from random_gb300 import build, capi, segy, synth
    from random_gb300.migration import Migration
    build.build()
    dev = torch.device("cuda", 0)
    counts = synth.offset_bin_counts(64, 15000.0, 2000, 40000, seed=4)
    mdl = synth.offset_bins_model(counts, ns=1001, dt=0.004, nx=160, ny=160, bin_m=12.5, aperture=1500.0,
                                  n_refl=8, n_diff=200, freq=25.0, mode=capi.MODE_REFERENCE, aa_cutoff=1e6)
    s = mdl.survey
    d_hdr = torch.from_numpy(np.ascontiguousarray(segy.headers_be(s.headers))).to(dev)
    d_smp = synth.synthesize_torch(mdl, device=dev)
    torch.cuda.synchronize()
    block = args.traces_per_step if args.traces_per_step != STEP_TRACES else 120_000
    nblocks = s.ntr // block
    m = Migration(dict(s.params, precision=capi.PREC_BF16_KAHAN), s.velocity)
    stream = torch.cuda.Stream(device=dev)
    m.set_stream(stream.cuda_stream)
    m.set_launch(persistent=1, graph=1)
    cfg, tune_ms = m.autotune(d_hdr.data_ptr(), d_smp.data_ptr(), 8000)
    m.set_launch(**dict(cfg, persistent=1, graph=1))
    row = 1001 * 4

    def step(i):
        b = i % nblocks
        m.add_traces_device(d_hdr.data_ptr() + b * block * 240, d_smp.data_ptr() + b * block * row, block)

    mark = {}
    elapsed, clk = _timed_steps(step, args.warmup, args.steps, stream,
                                after_warmup=lambda: mark.setdefault("p0", m.pairs()))
    m.synchronize()
    pairs_timed = m.pairs() - mark["p0"]
    line = {"workload": "offset-bins", "metric": METRIC, "value": round(pairs_timed / elapsed / 1e9, 4),
            "unit": UNIT, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(elapsed / args.steps * 1e3, 3), "dtype": "bf16 store, f32 compute",
            "config": {"bins": 64, "traces": int(s.ntr), "traces_per_step": block, "ns": 1001,
                       "image": "160x160x64x1001", "autotuned": cfg, "launch": m.launch_config(),
                       "autotune_ms": round(tune_ms, 3)},
            "pairs_per_step": pairs_timed / args.steps, "clocks": clk}
    print(json.dumps(line), flush=True)


def run_line(args):
    """The 2-D line: 200 CMPs x 48 offsets = 9,600 traces, 1001 samples at
    4 ms, 48 offset classes x 200 columns, reference operator (bit-exact
    accumulators).  The launch configuration is chosen by kpstm_autotune on
    the line itself (a fresh context), as a job loop would on its first block.
    A step images the whole line once (1.61e9 pairs) from device-resident
    traces."""
    import torch
    from random_gb300 import build, segy, synth
    from random_gb300.migration import Migration
    build.build()
    dev = torch.device("cuda", 0)
    s = synth.line2d()
    d_hdr = torch.from_numpy(np.ascontiguousarray(segy.headers_be(s.headers))).to(dev)
    d_smp = torch.from_numpy(np.ascontiguousarray(s.samples)).to(dev)
    m = Migration(s.params, s.velocity)
    stream = torch.cuda.Stream(device=dev)
    m.set_stream(stream.cuda_stream)
    cfg, tune_ms = m.autotune(d_hdr.data_ptr(), d_smp.data_ptr(), s.ntr)

    def step(i):
        m.add_traces_device(d_hdr.data_ptr(), d_smp.data_ptr(), s.ntr)

    mark = {}
    elapsed, clk = _timed_steps(step, args.warmup, args.steps, stream,
                                after_warmup=lambda: mark.setdefault("p0", m.pairs()))
    m.synchronize()
    pairs = m.pairs() - mark["p0"]
    line = {"workload": "line", "metric": METRIC, "value": round(pairs / elapsed / 1e9, 4), "unit": UNIT,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(elapsed / args.steps * 1e3, 3),
            "dtype": "f32", "config": {"traces": int(s.ntr), "ns": 1001, "image": "200x1x48x1001",
                                       "mode": "reference (bit-exact)", "launch": cfg,
                                       "autotune_ms": round(tune_ms, 3)},
            "pairs_per_step": pairs / args.steps, "clocks": clk}
    print(json.dumps(line), flush=True)


def run_lsm(args):
    """Least-squares operator pair on 250,000 traces (ns = 751 at 4 ms,
    offsets U(0, 3000 m), random azimuths) and a 200 x 200 x 751 model at
    25 m, aperture 3000 m, full physics: a step is one demigration d = L m
    plus one migration L^T d (the work of one CG iteration), BF16 data."""
    import torch
    from random_gb300 import build, capi, synth
    from random_gb300.migration import Migration
    build.build()
    dev = torch.device("cuda", 0)
    ntr = args.survey_traces if args.survey_traces != SURVEY_TRACES else 250_000
    mdl = synth.patch3d_model(ntr, ns=751, dt=0.004, nx=200, ny=200, bin_m=25.0, max_offset=3000.0, n_refl=12,
                              n_diff=100, freq=25.0, aperture=3000.0, seed=5, mode=capi.MODE_FULL,
                              output=capi.OUT_STACK)
    s = mdl.survey
    m = Migration(dict(s.params, precision=capi.PREC_BF16_KAHAN), s.velocity)
    stream = torch.cuda.Stream(device=dev)
    m.set_stream(stream.cuda_stream)
    m.lsm_geometry(s.headers)
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    model = torch.randn(*m.shape, device=dev, generator=g)
    data = torch.empty((ntr, 751), device=dev)
    torch.cuda.synchronize()
    t = {"fwd": 0.0, "adj": 0.0}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]

    def step(i):
        ev[0].record(stream)
        m.lsm_forward(model.data_ptr(), data.data_ptr())
        ev[1].record(stream)
        m.lsm_adjoint(data.data_ptr(), model.data_ptr())
        ev[2].record(stream)
        model.mul_(1.0 / (model.abs().max() + 1e-30))  # keep magnitudes bounded between steps
        if i >= args.warmup:
            torch.cuda.synchronize()
            t["fwd"] += ev[0].elapsed_time(ev[1]) / 1e3
            t["adj"] += ev[1].elapsed_time(ev[2]) / 1e3

    with torch.cuda.stream(stream):
        elapsed, clk = _timed_steps(step, args.warmup, args.steps, stream)
    pairs_app = m.lsm_pairs()
    line = {"workload": "lsm-operator-pair", "metric": METRIC,
            "value": round(2 * pairs_app * args.steps / (t["fwd"] + t["adj"]) / 1e9, 4), "unit": UNIT,
            "steps": args.steps, "warmup": args.warmup, "dtype": "bf16 data, f32 compute",
            "forward_gpairs_s": round(pairs_app * args.steps / t["fwd"] / 1e9, 4),
            "adjoint_gpairs_s": round(pairs_app * args.steps / t["adj"] / 1e9, 4),
            "pairs_per_application": pairs_app,
            "config": {"traces": ntr, "ns": 751, "model": "200x200x751", "aperture_m": 3000.0},
            "clocks": clk}
    if args.dot_test:
        # adjointness at this size: |<L m, d> - <m, L^T d>| for seeded random m, d
        gg = torch.Generator(device=dev)
        gg.manual_seed(11)
        mv = torch.randn(*m.shape, device=dev, generator=gg)
        dv = torch.randn((ntr, 751), device=dev, generator=gg)
        Lm = torch.empty_like(dv)
        Ltd = torch.empty_like(mv)
        m.lsm_forward(mv.data_ptr(), Lm.data_ptr())
        m.lsm_adjoint(dv.data_ptr(), Ltd.data_ptr())
        torch.cuda.synchronize()
        a_ = float((Lm.double() * dv.double()).sum())
        b_ = float((mv.double() * Ltd.double()).sum())
        line["dot_test"] = {"rel": abs(a_ - b_) / abs(a_),
                            "rel_to_norms": abs(a_ - b_) / float(Lm.double().norm() * dv.double().norm())}
    if args.cg_iters > 0:
        # least-squares migration of the survey's own events (bf16 data vectors,
        # FP64 CG scalars): time and residual history of --cg-iters iterations
        from random_gb300 import synth as _s
        d_obs = _s.synthesize_torch(mdl, device=dev)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        resid = m.lsm_cg(d_obs.data_ptr(), args.cg_iters, model.data_ptr())
        e1.record(stream)
        torch.cuda.synchronize()
        secs = e0.elapsed_time(e1) / 1e3
        line["cg"] = {"iterations": args.cg_iters, "seconds": round(secs, 3),
                      "applications": 2 * args.cg_iters,
                      "residual_rel": [round(float(r / resid[0]), 6) for r in resid]}
    if args.lsm_accuracy > 0:
        line["lsm_accuracy"] = _lsm_accuracy(args, mdl, m, stream, dev)
    print(json.dumps(line), flush=True)


def _lsm_accuracy(args, mdl, m16, stream, dev):
    """BF16-stored least-squares migration against FP32-stored CGLS of the
    same data (FP64 dot products and step lengths in both; the FP32 solver
    matches the FP64 oracle's CGLS to ~1e-6 relative where the oracle runs),
    and the wall time of each against one plain FP32 migration of the same
    survey (full mode: ingest, tap tables, imaging, finishing).  CGLS starts
    from m = 0, so the iterate after k iterations comes from a k-iteration
    run: each k is timed on its own."""
    import numpy as np
    import torch
    from random_gb300 import capi, segy, synth
    from random_gb300.migration import Migration
    s = mdl.survey
    d_obs = synth.synthesize_torch(mdl, device=dev)
    m32 = Migration(dict(s.params, precision=capi.PREC_FP32), s.velocity)
    m32.set_stream(stream.cuda_stream)
    m32.lsm_geometry(s.headers)
    x16 = torch.empty(*m16.shape, device=dev)
    x32 = torch.empty_like(x16)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    # plain FP32 migration of the same traces (second of two runs)
    mp = Migration(dict(s.params, precision=capi.PREC_FP32), s.velocity)
    mp.set_stream(stream.cuda_stream)
    hdr_be = torch.from_numpy(np.ascontiguousarray(segy.headers_be(s.headers), dtype=np.int32)).to(dev)
    img = torch.empty(*mp.shape, device=dev)
    t_plain = 0.0
    for _ in range(2):
        mp.reset()
        t_plain = timed(lambda: (mp.add_traces_device(hdr_be.data_ptr(), d_obs.data_ptr(), s.ntr),
                                 mp.finish_device(img.data_ptr())))
    err, t16, t32 = [], [], []
    for k in range(1, args.lsm_accuracy + 1):
        t16.append(timed(lambda: m16.lsm_cg(d_obs.data_ptr(), k, x16.data_ptr())))
        t32.append(timed(lambda: m32.lsm_cg(d_obs.data_ptr(), k, x32.data_ptr())))
        err.append(float((x16.double() - x32.double()).norm() / x32.double().norm()))
    hit = next((k + 1 for k, e in enumerate(err) if e <= 1e-3), None)
    return {"reference": "FP32-stored CGLS, FP64 scalars", "iterations": list(range(1, args.lsm_accuracy + 1)),
            "rel_l2_bf16_vs_fp32": [round(e, 7) for e in err],
            "bf16_seconds": [round(t, 3) for t in t16], "fp32_seconds": [round(t, 3) for t in t32],
            "plain_fp32_migration_seconds": round(t_plain, 3),
            "bf16_seconds_over_plain": [round(t / t_plain, 3) for t in t16],
            "last_iteration_within_1e-3": max([k + 1 for k, e in enumerate(err) if e <= 1e-3], default=None),
            "first_iteration_within_1e-3": hit}


# ----------------------------------------------------------- reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return
    cores = host_cores()
    vals, pairs_t, secs_t = [], 0, 0.0
    for i in range(args.warmup + args.steps):
        pairs, secs, nslab = cpu_sample(args.ref_traces, cores)
        if i >= args.warmup:
            vals.append(pairs / secs / 1e9)
            pairs_t += pairs
            secs_t += secs
    value = pairs_t / secs_t / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(secs_t / args.steps * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (same seeded survey as the GPU arm)",
        "config": {"workload": "3-D PSTM, 1e6 traces x 1501 samples @ 2 ms, 400x400x1501 stack image at "
                               "25 m, aperture 3000 m (the reference's own operator: nearest-sample T, "
                               "fixed triangle)", "sample_traces": args.ref_traces, "slabs": nslab},
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": nslab, "kind": "reference",
                         "sample": f"{nslab} of 400 one-iline slabs x first {args.ref_traces} traces per step"},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--traces-per-step", type=int, default=STEP_TRACES)
    ap.add_argument("--survey-traces", type=int, default=SURVEY_TRACES,
                    help="traces synthesised on the device (smaller only for profiling captures)")
    ap.add_argument("--cpu-traces", type=int, default=3000)
    ap.add_argument("--ref-traces", type=int, default=1500)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cg-iters", type=int, default=0, help="lsm workload: also time this many CG iterations")
    ap.add_argument("--dot-test", action="store_true", help="lsm workload: also run the dot-product test")
    ap.add_argument("--lsm-accuracy", type=int, default=0,
                    help="lsm workload: BF16 vs FP32 CGLS iterates and times for 1..N iterations, "
                         "against one plain FP32 migration of the same survey")
    ap.add_argument("--autotune", type=int, default=0,
                    help="survey workload: autotune the launch on this many traces before timing (0: default launch)")
    ap.add_argument("--precision", choices=["fp32", "bf16"], default="fp32",
                    help="trace storage of the survey workload (bf16: per-trace scale, Kahan sums)")
    ap.add_argument("--workload", choices=["survey", "offset-bins", "lsm", "line"], default="survey",
                    help="survey: the bench line; offset-bins / lsm / line: further measurements (1 GPU)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "offset-bins":
        run_offset_bins(args)
        return
    if args.workload == "lsm":
        run_lsm(args)
        return
    if args.workload == "line":
        run_line(args)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
