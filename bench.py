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
def survey_model(rank: int = 0, ntr: int = SURVEY_TRACES, image: int = NX):
    from random_gb300 import multirank, synth
    # each rank: its own 10 km x 10 km slab (x shifted), same statistics;
    # image < 400 (profiling captures): a smaller patch at the same sampling
    return synth.patch3d_model(ntr, ns=NS, dt=DT, nx=image, ny=image, bin_m=25.0, max_offset=4000.0,
                               n_refl=8, n_diff=200, freq=30.0, aperture=3000.0, aa_cutoff=100.0,
                               seed=2 + rank, mode=1, output=1,
                               x_shift=multirank.weak_scaling_shift(rank, 20000.0))


def algorithmic_bytes_per_step(model, ntr_step: int, row_floats: int) -> int:
    """Compulsory bytes of one imaging launch: the block's tap tables read
    once, geometry, the image accumulators (sums + counts) read and written
    once, and the velocity rows."""
    nx = model.survey.params["end_iline"] - model.survey.params["start_iline"]
    ny = model.survey.params["end_xline"] - model.survey.params["start_xline"]
    return ntr_step * row_floats * 4 + ntr_step * 32 + nx * ny * NS * 4 * 2 * 2 + nx * NS * 8



# ------------------------------------------------------------------ roofline
# Algorithmic operations of one pair (one pass of Kirchhoff.c:1374-1399),
# counted as FP32-pipe lane operations (an FMA, an add, a compare, a shared
# load each count 1) and MUFU operations:
#   reference mode: 2 FMA for the two DSR arguments, 2 square roots, 1 add,
#   1 multiply by 1/dt, 1 floor, 3 tap loads, 3 tap adds, 1 accumulate,
#   1 fold increment, 1 compare = 14 FP32 + 2 MUFU;
#   full mode adds ~4 FMA (interpolation, weights) and 1 MUFU (1/Lf).
OPS_PER_PAIR = {"reference": (14, 2), "full": (18, 3), "full_bf16": (18, 3)}
# which committed ncu summary holds the figures of each kernel flavour
PROFILE_OF = {"full": "k_image_full_3d_ncu.md", "full_bf16": "k_image_full_3d_ncu.md",
              "reference": "k_image_line_ncu.md"}
KERNEL_SOURCES = ["random_gb300/csrc/kpstm_kernels.cuh", "random_gb300/csrc/kpstm_device.cuh"]


def kernel_source_hash() -> str:
    import hashlib
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        h.update((ROOT / f).read_bytes())
    return h.hexdigest()[:16]


def profile_constants(name: str) -> dict | None:
    """The machine-readable block of a committed ncu summary: the JSON code
    block under its 'Bench constants' heading (figures of one capture, the
    launch it was taken on and the kernel-source hash at capture time)."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    text = p.read_text()
    i = text.find("## Bench constants")
    if i < 0:
        return None
    j = text.find("```json", i)
    k = text.find("```", j + 7)
    if j < 0 or k < 0:
        return None
    return json.loads(text[j + 7:k])


def imaging_roofline(pairs_per_launch, t_launch, b_alg, clk, peaks, dev, launch_cfg, flavour,
                     table_rows=None, row_bytes=None, image_columns=None) -> dict:
    """Roofline of one imaging launch.  The binding resource is the FP32
    lane-issue rate for the algorithmic op count (no tensor work; the kernel
    moves ~1e-3 byte per pair): achieved = ops/pair x pairs/s, peak = SMs x
    128 FP32 lanes x the SM clock sampled during the timed region.  HBM,
    MUFU, issue slots and L2 are sub-fields; the ncu-derived figures come
    from the committed summary of the same kernel flavour and are flagged
    stale when the kernel sources or the launch differ from the capture."""
    import torch
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = clk.get("sm_mhz") or peaks["sm_max_mhz"]
    rate = pairs_per_launch / t_launch
    f32, mufu = OPS_PER_PAIR[flavour]
    peak_ops = sms * 128 * mhz * 1e6
    achieved = f32 * rate
    out = {"bound": "fp32 lane issue (algorithmic ops)", "achieved": round(achieved / 1e12, 3),
           "peak": round(peak_ops / 1e12, 3), "unit": "TFLOP/s", "frac": round(achieved / peak_ops, 4),
           "ops_per_pair": {"fp32": f32, "mufu": mufu, "note": "lane operations; an FMA counts 1"},
           "peak_basis": f"{sms} SMs x 128 FP32 lanes x {mhz:.0f} MHz (sampled)",
           "launch_ms": round(t_launch * 1e3, 3), "pairs_per_launch": pairs_per_launch,
           "hbm": {"achieved": round(b_alg / t_launch / 1e9, 3), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                   "frac": round(b_alg / t_launch / 1e9 / peaks["hbm_gbs"], 6), "peak_source": peaks["source"],
                   "algorithmic_bytes_per_launch": b_alg},
           "traffic": None}
    pc = profile_constants(PROFILE_OF[flavour])
    if pc is None:
        out["profile"] = None
        return out
    cur = kernel_source_hash()
    same_launch = all(pc.get("launch", {}).get(k) == launch_cfg.get(k)
                      for k in ("tile_px", "samples_per_lane", "persistent", "ctas_per_sm"))
    ipp = pc["warp_instructions"] / pc["pairs"]
    issue_peak = sms * 4 * mhz * 1e6
    out["issue_slots"] = {"instr_per_32_pairs": round(32 * ipp, 2),
                          "frac": round(rate * ipp / issue_peak, 4),
                          "ncu_issue_active": pc.get("issue_active")}
    out["mufu"] = {"ops_per_pair": mufu, "ncu_xu_pipe": pc.get("xu_pipe")}
    if pc.get("lts_bytes") is not None:
        out["l2"] = {"achieved": round(pc["lts_bytes"] / pc["pairs"] * rate / 1e9, 1), "unit": "GB/s",
                     "bytes_per_pair": round(pc["lts_bytes"] / pc["pairs"], 5),
                     "ncu_lts_throughput": pc.get("lts_throughput")}
    if pc.get("dram_bytes") is not None:
        # fixed part (accumulators, velocity rows) scaled by the image columns,
        # table part by the rows staged
        fixed, tab = pc["dram_bytes"], 0
        if table_rows and pc.get("table_rows") and row_bytes:
            fixed -= pc["table_rows"] * row_bytes
            tab = table_rows * row_bytes
        if image_columns and pc.get("image_columns"):
            fixed *= image_columns / pc["image_columns"]
        out["traffic"] = round(fixed + tab)
        out["traffic_source"] = (f"ncu dram bytes of the capture in profiles/{PROFILE_OF[flavour]} "
                                 f"({pc.get('case', '')}), table part scaled to this launch")
    out["profile"] = {"file": f"profiles/{PROFILE_OF[flavour]}", "kernel": pc.get("kernel"),
                      "stale": pc.get("source_sha256") != cur or not same_launch,
                      "source_sha256": cur, "captured_sha256": pc.get("source_sha256")}
    return out

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
    model = survey_model(rank, args.survey_traces, args.image)
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
    roofline = imaging_roofline(pairs / launches, t_launch, b_alg, clk, peaks, dev, launch_cfg,
                                "full_bf16" if args.precision == "bf16" else "full",
                                table_rows=block, row_bytes=row_floats * 4, image_columns=args.image * args.image)
    roofline["image_kernel_share"] = round(prof["image_ms"] / (prof["image_ms"] + prof["prep_ms"]), 4)
    # live pairs: those whose traveltime falls inside the trace (the fold
    # counts), against all counted (trace, column, sample) pairs so far
    _, fold = m.accumulators()
    live = float(np.sum(fold.astype(np.float64) - 1.0))
    live_fraction = live / max(1, m.pairs())
    del fold
    # the same roofline over live pairs only: the kernel skips dead pairs
    # (whole trace windows left out of a tile's list, masked halves), so the
    # algorithmic ops of the counted pairs overstate the work done
    roofline["live_pairs"] = {"fraction": round(live_fraction, 4),
                              "achieved": round(roofline["achieved"] * live_fraction, 3),
                              "frac": round(roofline["frac"] * live_fraction, 4)}
    del m

    # -------- the reference's own operator (nearest-sample traveltime, fixed
    # triangle, unit weight: the mode that reproduces Kirchhoff.c bit for bit)
    # on the same survey and blocks, so that the CPU baseline, which runs that
    # operator, has a same-operator GPU figure beside the full-physics headline
    same_op = None
    if not args.no_cpu:
        mr = Migration(dict(prm, mode=capi.MODE_REFERENCE), s.velocity)
        mr.set_stream(stream.cuda_stream)
        for i in range(2):
            step_m = (i % nblocks) * block
            mr.add_traces_device(d_hdr.data_ptr() + step_m * 240, d_smp.data_ptr() + step_m * row_bytes, block)
        mr.synchronize()
        pr0 = mr.pairs()
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r0.record(stream)
        nref = min(args.steps, 3)
        for i in range(nref):
            step_m = ((2 + i) % nblocks) * block
            mr.add_traces_device(d_hdr.data_ptr() + step_m * 240, d_smp.data_ptr() + step_m * row_bytes, block)
        r1.record(stream)
        torch.cuda.synchronize()
        same_op = {"gpu_reference_mode_gpairs_s": round((mr.pairs() - pr0) / (r0.elapsed_time(r1) / 1e3) / 1e9, 4),
                   "steps": nref, "launch": mr.launch_config(),
                   "note": "the reference operator on the GPU (accumulators bit for bit equal to Kirchhoff.c's), "
                           "same survey and blocks as the headline"}
        del mr

    # -------- e2e through the C ABI from pinned host memory
    e2e = None
    if not args.no_e2e:
        nb = min(nblocks, 4)
        h_hdr = torch.from_numpy(hdr_be[:nb * block]).pin_memory()
        h_smp = d_smp[:nb * block].cpu().pin_memory()
        m2 = Migration(prm, s.velocity)
        m2.set_launch(**launch_cfg)
        out = torch.empty((args.image, args.image, 1, NS), dtype=torch.float32).pin_memory()
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

    if same_op and cpu:
        same_op["ratio_to_cpu_baseline"] = round(same_op["gpu_reference_mode_gpairs_s"] / cpu["value"], 1)
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
            "live_pair_fraction": round(live_fraction, 4),
            "same_operator": same_op,
            "trace_storage": {"bytes_per_trace": NS * (2 if args.precision == "bf16" else 4) +
                              (4 if args.precision == "bf16" else 0),
                              "gb_per_s": round(block * (NS * (2 if args.precision == "bf16" else 4)) /
                                                (elapsed_max / args.steps) / 1e9, 4),
                              "note": "stored trace bytes of a step / step time"},
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


def cpu_line(nprocs: int, opt: str = "-O3"):
    """The reference's kirchhoff() on the whole 2-D line (9,600 traces): the compiled
    Kirchhoff.c (MPI/FFTW stand-ins) with its image cut into nprocs slabs
    along the line (number_mpi_jobsX = nprocs, Kirchhoff.c:280-300), one
    process per slab, all started together; every slab reads all traces
    (Kirchhoff.c:1276).  Returns the wall seconds until the last ends."""
    from oracle import refbuild
    from random_gb300 import synth
    s = synth.line2d()
    work = Path(tempfile.mkdtemp(prefix="kline_"))
    try:
        s.write_files(work / "data.segy", work / "vel.segy")
        cfg = refbuild.RefConfig(**s.ref_config(jobs_x=nprocs, jobs_y=1))
        binary = refbuild.compile(cfg, opt=opt, tag=f"line{nprocs}")
        (work / "run" / "image_dir").mkdir(parents=True, exist_ok=True)
        for name in ("data.segy", "vel.segy"):
            os.symlink(work / name, work / "run" / name)
        t0 = time.perf_counter()
        procs = [subprocess.Popen([str(binary)], cwd=work / "run", stdout=subprocess.DEVNULL,
                                  stderr=subprocess.DEVNULL, stdin=subprocess.DEVNULL,
                                  env=dict(os.environ, KPSTM_REF_RANK=str(j), KPSTM_REF_SIZE=str(nprocs)))
                 for j in range(nprocs)]
        for p in procs:
            p.wait()
        secs = time.perf_counter() - t0
        if any(p.returncode for p in procs):
            raise RuntimeError("reference rank failed")
    finally:
        shutil.rmtree(work, ignore_errors=True)
    return secs


def run_line(args):
    """Config 1, the 2-D line: 200 CMPs x 48 offsets = 9,600 traces, 1001
    samples at 4 ms, 48 offset classes x 200 columns, reference operator
    (accumulators bit-exact to the reference).  The launch is the one
    kpstm_autotune picks on the line (8 x 1 tiles, K = 8, 3 CTAs per SM; with
    --autotune N > 0 the autotuner runs on the line itself, as a job loop
    would on its first block).  A step images the whole line once
    (1.61e9 pairs) from device-resident traces.  e2e: the same job through
    kpstm_add_traces from pinned host buffers and kpstm_finish (image and
    fold to host) per step.  CPU: the compiled reference on one rank over
    the whole line (the config's "1 MPI rank"), and on all host cores with
    its own slab decomposition."""
    import torch
    from random_gb300 import build, segy, synth
    from random_gb300.migration import Migration
    build.build()
    dev = torch.device("cuda", 0)
    peaks = load_peaks()
    s = synth.line2d()
    hdr_np = np.ascontiguousarray(segy.headers_be(s.headers))
    d_hdr = torch.from_numpy(hdr_np).to(dev)
    d_smp = torch.from_numpy(np.ascontiguousarray(s.samples)).to(dev)
    m = Migration(s.params, s.velocity)
    stream = torch.cuda.Stream(device=dev)
    m.set_stream(stream.cuda_stream)
    if args.autotune <= 0:
        # the autotuner's usual choice on this line: 8 x 1 tiles, K = 8, 3 CTAs per SM, grid launch
        m.set_launch(tile_px=8, samples_per_lane=8, persistent=0, ctas_per_sm=3)
        cfg, tune_ms = m.launch_config(), 0.0
    else:
        cfg, tune_ms = m.autotune(d_hdr.data_ptr(), d_smp.data_ptr(), s.ntr)

    def step(i):
        m.add_traces_device(d_hdr.data_ptr(), d_smp.data_ptr(), s.ntr)

    for i in range(args.warmup):
        step(i)
    m.synchronize()
    p0 = m.pairs()
    m.profile(True)
    m.profile_read()
    # each step timed on its own, L2 flushed (a 512 MB write) between steps
    flush = torch.empty(128 << 20, dtype=torch.float32, device=dev)
    clocks = ClockSampler(0)
    clocks.start()
    elapsed = 0.0
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(args.warmup + i)
        e1.record(stream)
        torch.cuda.synchronize()
        elapsed += e0.elapsed_time(e1) / 1e3
    clk = clocks.stop()
    del flush
    mark = {"p0": p0}
    m.synchronize()
    prof = m.profile_read()
    m.profile(False)
    pairs = m.pairs() - mark["p0"]
    launch_cfg = m.launch_config()
    launches = max(1, int(prof["image_launches"]))
    t_launch = prof["image_ms"] / 1e3 / launches
    ncol, ncls, ns = 200, 48, 1001
    row = ns + 1 + 8  # tap row (reference mode) + geometry header, floats
    b_alg = s.ntr * row * 4 + s.ntr * 32 + ncol * ncls * ns * 4 * 2 * 2 + ncol * ns * 8
    roofline = imaging_roofline(pairs / args.steps, t_launch, b_alg, clk, peaks, dev, launch_cfg, "reference")
    roofline["image_kernel_share"] = round(prof["image_ms"] / (elapsed * 1e3), 4)
    del m

    # e2e: host buffers in, finished image and fold out, every step a whole job
    h_hdr = torch.from_numpy(hdr_np).pin_memory()
    h_smp = torch.from_numpy(np.ascontiguousarray(s.samples)).pin_memory()
    out = torch.empty((ncol, 1, ncls, ns), dtype=torch.float32).pin_memory()
    fold = torch.empty_like(out).pin_memory()
    m2 = Migration(s.params, s.velocity)
    m2.set_launch(**launch_cfg)
    for _ in range(args.warmup):
        m2.reset()
        m2.add_traces_ptr(h_hdr.data_ptr(), h_smp.data_ptr(), s.ntr)
        m2.finish_ptr(out.data_ptr(), fold.data_ptr())
    t0 = time.perf_counter()
    pe = 0
    for _ in range(args.steps):
        m2.reset()
        p0 = m2.pairs()
        m2.add_traces_ptr(h_hdr.data_ptr(), h_smp.data_ptr(), s.ntr)
        m2.finish_ptr(out.data_ptr(), fold.data_ptr())
        pe += m2.pairs() - p0
    t_e2e = time.perf_counter() - t0
    del m2
    e2e = {"value": round(pe / t_e2e / 1e9, 4), "unit": UNIT,
           "h2d_bytes_per_step": int(hdr_np.nbytes + s.samples.nbytes),
           "d2h_bytes_per_step": int(out.numel() * 4 * 2),
           "note": "per step: kpstm_reset, kpstm_add_traces from pinned host buffers, kpstm_finish "
                   "(image and fold to host); wall clock"}

    cpu = None
    if not args.no_cpu:
        t1 = cpu_line(1)
        cores = host_cores()
        tn = cpu_line(cores)
        ppj = pe / args.steps
        cpu = {"value": round(ppj / t1 / 1e9, 4), "unit": UNIT, "cores": 1, "kind": "reference",
               "sample": f"the whole line (9,600 traces, {ppj:.4g} pairs) by the reference kirchhoff() "
                         f"(-O3 -ffast-math, MPI/FFTW stand-ins) on one rank: {t1:.2f} s",
               "all_cores": {"value": round(ppj / tn / 1e9, 4), "cores": cores,
                             "sample": f"the same line cut into {cores} slabs (number_mpi_jobsX = {cores}), "
                                       f"one rank per core: {tn:.2f} s"}}
    line = {"workload": "line", "metric": METRIC, "value": round(pairs / elapsed / 1e9, 4), "unit": UNIT,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(elapsed / args.steps * 1e3, 3), "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded 2-D line: 20 point scatterers, 25 Hz Ricker, 20 dB noise)",
            "config": {"workload": "2-D line, 200 CMPs x 48 offsets = 9,600 traces x 1001 samples "
                                   "@ 4 ms, 200 x 48 x 1001 offset gathers, aperture 1500 m, reference operator",
                       "traces": int(s.ntr), "launch": cfg, "autotune_ms": round(tune_ms, 3),
                       "l2": "flushed between timed steps (512 MB write); each step timed alone"},
            "pairs_per_step": pairs / args.steps, "gpu_launches": int(prof["image_launches"] + prof["other_launches"]),
            "roofline": roofline, "e2e": e2e, "cpu_baseline": cpu, "clocks": clk}
    print(json.dumps(line), flush=True)


def _progress(line: dict, stage: str) -> None:
    """The least-squares line so far, on stderr (a long run that is cut
    short still leaves its finished stages)."""
    print(json.dumps({"progress": stage, **line}), file=sys.stderr, flush=True)


def lsm_problem(ntr: int, nx: int = 200, ny: int = 200, ns: int = 751, n_scat: int = 100, seed: int = 5):
    """Config 5: the acquisition (synth.lsm_survey_model) and the seeded
    reflectivity model m_true [nx, ny, 1, ns] (12 dipping reflectors and
    n_scat scatterers); the data are d = L m_true plus 10 dB Gaussian noise,
    made by the caller with its own L."""
    from random_gb300 import synth
    mdl = synth.lsm_survey_model(ntr, nx=nx, ny=ny, ns=ns, seed=seed)
    p = mdl.survey.params
    m_true = synth.reflectivity_model(nx, ny, ns, float(p["dt"]), 25.0, n_refl=12, n_scat=n_scat, seed=seed,
                                      x0=p["start_iline"] * 25.0)
    return mdl, m_true


LSM_SNR_DB = 10.0


def lsm_cpu_subproblem(args, dev, stream):
    """The FP64-oracle leg of the least-squares workload (bench's CPU
    baseline for it): a 16 x 16-column crop of the 200 x 200 x 751 model with 1,000
    traces of the same acquisition statistics and 4 scatterers (the full
    survey's scatterer density), d = L m_true (FP64 oracle) + 10 dB noise,
    rounded to float32 for every solver.  The oracle's FP64 CGLS (timed on
    the host cores) is the reference iterate for each k; the GPU's BF16- and
    FP32-stored CGLS of the same data are compared with it at equal k."""
    import torch
    from oracle import oracle
    from random_gb300 import capi
    from random_gb300.migration import Migration
    mdl, m_true = lsm_problem(1000, nx=16, ny=16, n_scat=4, seed=7)
    s = mdl.survey
    d = oracle.lsm_apply(s, 1, m_true)
    rng = np.random.default_rng(7)
    d += rng.normal(0.0, float(np.sqrt(np.mean(d ** 2))) / 10.0 ** (LSM_SNR_DB / 20.0), d.shape)
    d32 = d.astype(np.float32)
    niter = args.cg_iters
    t0 = time.perf_counter()
    x64, res64 = oracle.cgls(s, d32.astype(np.float64), niter)
    t_cpu = time.perf_counter() - t0
    dd = torch.from_numpy(d32).to(dev)
    out = {}
    for name, prec in (("bf16", capi.PREC_BF16_KAHAN), ("fp32", capi.PREC_FP32)):
        with Migration(dict(s.params, precision=prec), s.velocity) as mg:
            mg.set_stream(stream.cuda_stream)
            mg.lsm_geometry(s.headers)
            xm = torch.empty(mg.shape, dtype=torch.float32, device=dev)
            snaps = []
            mg.lsm_cg(dd.data_ptr(), niter, xm.data_ptr(),
                      monitor=lambda k, ptr, res: snaps.append(xm.to("cpu", copy=True).numpy()) and False)
            out[name] = [float(np.linalg.norm(a.astype(np.float64).reshape(b.shape) - b) / np.linalg.norm(b))
                         for a, b in zip(snaps, x64)]
    pairs = 2 * niter * 1000 * 16 * 16 * 751  # upper bound: every (trace, column, sample) of the crop
    return {"problem": "16 x 16 columns of the 200 x 200 x 751 model (25 m, 4 ms), 1,000 traces (offsets "
                       "U(0, 3000 m), random azimuths, midpoints over the crop), 12 dipping reflectors + 4 "
                       "scatterers, d = L m_true (FP64) + 10 dB noise, float32 data",
            "rel_l2_vs_fp64": {k: [round(e, 8) for e in v] for k, v in out.items()},
            "fp64_residual_rel": [round(float(r / res64[0]), 6) for r in res64],
            "fp64_cgls_seconds": round(t_cpu, 2), "cores": host_cores(),
            "fp64_pairs_bound": pairs}


def run_lsm(args):
    """Least-squares Kirchhoff migration: a 200 x 200 x 751
    reflectivity model (25 m, 4 ms; 12 dipping reflectors + 100 scatterers),
    d = L m_true on 250,000 traces (offsets U(0, 3000 m), random azimuths,
    751 samples) plus 10 dB Gaussian noise, aperture 3000 m, full physics;
    --cg-iters (20) CG iterations in BF16-stored / FP32-accumulated form with
    FP64 scalars.  Reports the operator rates (L, L^T), the dot-product test
    and --fd-dirs finite-difference checks at this size, the CG wall time and
    residual history, one plain FP32 migration of the same survey, the
    BF16 iterate's error against FP32-stored CGLS at full size
    (--lsm-ref-iters iterations) and against the FP64 oracle's CGLS on a
    sub-problem, and from these the wall time at which the BF16 iterate is
    first within 1e-3 of the FP64-oracle iterate of the same iteration, in
    plain migrations."""
    import torch
    from random_gb300 import build, capi, segy
    from random_gb300.migration import Migration
    build.build()
    dev = torch.device("cuda", 0)
    ntr = args.survey_traces if args.survey_traces != SURVEY_TRACES else 250_000
    mdl, m_true_np = lsm_problem(ntr)
    s = mdl.survey
    ns = s.ns
    stream = torch.cuda.Stream(device=dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def timed(fn):
        a, b = ev(), ev()
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3

    m16 = Migration(dict(s.params, precision=capi.PREC_BF16_KAHAN), s.velocity)
    m16.set_stream(stream.cuda_stream)
    m16.lsm_geometry(s.headers)
    m_true = torch.from_numpy(m_true_np).to(dev)
    d_obs = torch.empty((ntr, ns), device=dev)
    model = torch.empty_like(m_true)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        # d = L m_true + 10 dB Gaussian noise (seeded)
        m16.lsm_forward(m_true.data_ptr(), d_obs.data_ptr())
        m16.lsm_adjoint(d_obs.data_ptr(), model.data_ptr())  # counts the pairs
        torch.cuda.synchronize()
        gen = torch.Generator(device=dev)
        gen.manual_seed(5)
        sigma = float(d_obs.double().pow(2).mean().sqrt()) / 10.0 ** (LSM_SNR_DB / 20.0)
        d_obs.add_(torch.randn(d_obs.shape, device=dev, generator=gen), alpha=sigma)
        torch.cuda.synchronize()
    pairs_app = m16.lsm_pairs()

    # operator rates: --steps (L, L^T) applications after --warmup on dense
    # seeded random vectors (what CG applies: its search directions and
    # residuals have no zero samples); L on the sparse reflectivity once
    # (zero model samples skip their pairs)
    gg = torch.Generator(device=dev)
    gg.manual_seed(11)
    mv = torch.randn(m_true.shape, device=dev, generator=gg)
    dv = torch.randn((ntr, ns), device=dev, generator=gg)
    Lm, Ltd = torch.empty_like(dv), torch.empty_like(mv)
    tf, ta = [], []
    clocks = None
    for i in range(args.warmup + args.steps):
        if i == args.warmup:
            clocks = ClockSampler(0)
            clocks.start()
        f = timed(lambda: m16.lsm_forward(mv.data_ptr(), Lm.data_ptr()))
        a = timed(lambda: m16.lsm_adjoint(dv.data_ptr(), Ltd.data_ptr()))
        if i >= args.warmup:
            tf.append(f)
            ta.append(a)
    clk = clocks.stop() if clocks else None
    t_sparse = timed(lambda: m16.lsm_forward(m_true.data_ptr(), Lm.data_ptr()))
    t_L, t_Lt = statistics.median(tf), statistics.median(ta)
    line = {"workload": "lsm",
            "metric": "BF16 LSM wall time to 1e-3 FP64-oracle image error, in plain FP32 migrations of the survey",
            "unit": "migrations", "higher_is_better": False,
            "dtype": "bf16 data/residual store, f32 compute, f64 CG scalars",
            "data": "synthetic: d = L m_true + 10 dB Gaussian noise (seeded)",
            "config": {"workload": "least-squares survey: 200x200x751 reflectivity (25 m, 4 ms), 12 dipping reflectors + 100 "
                                   "scatterers, 250,000 traces x 751 samples, offsets U(0, 3000 m), random "
                                   "azimuths, aperture 3000 m, full physics", "traces": ntr,
                       "cg_iterations": args.cg_iters},
            "pairs_per_application": pairs_app,
            "operators": {"L_seconds": round(t_L, 4), "Lt_seconds": round(t_Lt, 4),
                          "L_gpairs_s": round(pairs_app / t_L / 1e9, 2),
                          "Lt_gpairs_s": round(pairs_app / t_Lt / 1e9, 2), "samples": len(tf),
                          "vectors": "dense seeded random model and data",
                          "L_on_reflectivity_gpairs_s": round(pairs_app / t_sparse / 1e9, 2)},
            "clocks": clk}

    # dot-product test at full size: <L m, d> = <m, L^T d> for the same vectors
    with torch.cuda.stream(stream):
        m16.lsm_forward(mv.data_ptr(), Lm.data_ptr())
        m16.lsm_adjoint(dv.data_ptr(), Ltd.data_ptr())
    torch.cuda.synchronize()
    a_, b_ = float((Lm.double() * dv.double()).sum()), float((mv.double() * Ltd.double()).sum())
    line["dot_test"] = {"rel": abs(a_ - b_) / abs(a_), "bar": 1e-5,
                        "rel_to_norms": abs(a_ - b_) / float(Lm.double().norm() * dv.double().norm())}
    _progress(line, "operators, dot test")
    del dv, Ltd

    # finite-difference checks of the misfit gradient, J(m) = |L m - d|^2 / 2,
    # g = L^T (L m - d), central differences along --fd-dirs random directions
    if args.fd_dirs > 0:
        with torch.cuda.stream(stream):
            m16.lsm_forward(mv.data_ptr(), Lm.data_ptr())
            res = Lm - d_obs
            g = torch.empty_like(mv)
            m16.lsm_adjoint(res.data_ptr(), g.data_ptr())
            torch.cuda.synchronize()
            worst, rels = 0.0, []
            dm = torch.empty_like(mv)
            mp = torch.empty_like(mv)
            Lp = torch.empty_like(Lm)

            def J(x):
                m16.lsm_forward(x.data_ptr(), Lp.data_ptr())
                torch.cuda.synchronize()
                return 0.5 * float((Lp.double() - d_obs.double()).pow(2).sum())
            for k in range(args.fd_dirs):
                dm.normal_(generator=gg)
                h = 1e-2 * float(mv.norm()) / float(dm.norm())
                torch.add(mv, dm, alpha=h, out=mp)
                jp = J(mp)
                torch.add(mv, dm, alpha=-h, out=mp)
                jm = J(mp)
                fd = (jp - jm) / (2 * h)
                an = float((g.double() * dm.double()).sum())
                rels.append(abs(fd - an) / abs(an))
            line["fd_check"] = {"directions": args.fd_dirs, "max_rel": max(rels),
                                "median_rel": statistics.median(rels), "bar": 2e-3}
            _progress(line, "finite differences")
            del res, g, dm, mp, Lp
    del mv, Lm
    torch.cuda.empty_cache()

    # one plain FP32 migration of the same survey: ingest, tap tables, imaging, finishing
    mp_ = Migration(dict(s.params, precision=capi.PREC_FP32), s.velocity)
    mp_.set_stream(stream.cuda_stream)
    hdr_be = torch.from_numpy(np.ascontiguousarray(segy.headers_be(s.headers), dtype=np.int32)).to(dev)
    img = torch.empty(mp_.shape, device=dev)
    t_plain = []
    for _ in range(3):
        mp_.reset()
        t_plain.append(timed(lambda: (mp_.add_traces_device(hdr_be.data_ptr(), d_obs.data_ptr(), ntr),
                                      mp_.finish_device(img.data_ptr()))))
    t_plain = min(t_plain[1:])
    mp_.close()
    del img, hdr_be
    line["plain_fp32_migration_seconds"] = round(t_plain, 4)

    # CGLS: BF16-stored (timed, with the iterate after every iteration) and
    # FP32-stored (the full-size reference of the BF16 iterates)
    def solve(mg, niter, keep):
        snaps, marks = [], []
        e0 = ev()

        def mon(k, ptr, res):
            e = ev()
            e.record(stream)
            marks.append(e)
            if keep:
                with torch.cuda.stream(stream):
                    snaps.append(model.clone())
            return False
        with torch.cuda.stream(stream):
            e0.record(stream)
            resid = mg.lsm_cg(d_obs.data_ptr(), niter, model.data_ptr(), monitor=mon)
        torch.cuda.synchronize()
        return snaps, [e0.elapsed_time(e) / 1e3 for e in marks], resid

    refk = min(args.lsm_ref_iters, args.cg_iters)
    snaps16, tk, resid = solve(m16, args.cg_iters, refk > 0)
    line["cg"] = {"iterations": len(tk), "seconds": round(tk[-1], 3) if tk else 0.0,
                  "seconds_at_iteration": [round(t, 3) for t in tk],
                  "seconds_over_plain_at_iteration": [round(t / t_plain, 3) for t in tk],
                  "residual_rel": [round(float(r / resid[0]), 6) for r in resid],
                  "applications": 2 * len(tk)}
    _progress(line, "bf16 cg")
    m16.close()
    err_full = []
    if refk > 0:
        m32 = Migration(dict(s.params, precision=capi.PREC_FP32), s.velocity)
        m32.set_stream(stream.cuda_stream)
        m32.lsm_geometry(s.headers)
        snaps32, _, _ = solve(m32, refk, True)
        m32.close()
        err_full = [float((a.double() - b.double()).norm() / b.double().norm()) for a, b in zip(snaps16, snaps32)]
        line["bf16_vs_fp32_full_size"] = [round(e, 8) for e in err_full]
        _progress(line, "fp32 cg")
    del snaps16
    torch.cuda.empty_cache()

    sub = None
    if not args.no_cpu:
        sub = lsm_cpu_subproblem(args, dev, stream)
        line["fp64_subproblem"] = sub
        line["cpu_baseline"] = {"value": sub["fp64_cgls_seconds"], "unit": "s (FP64 oracle CGLS, sub-problem)",
                                "cores": sub["cores"], "kind": "port",
                                "sample": f"{args.cg_iters} CG iterations of the FP64 oracle on the 16 x 16-column, "
                                          f"1,000-trace sub-problem"}
    # BF16 iterate k is within 1e-3 of the FP64-oracle iterate when the full-size
    # BF16-vs-FP32 error plus the sub-problem's FP32-vs-FP64 gap is at most 1e-3
    # and the sub-problem's BF16-vs-FP64 error is too
    within = []
    for k in range(len(tk)):
        e = err_full[k] if k < len(err_full) else None
        gap = sub["rel_l2_vs_fp64"]["fp32"][k] if sub and k < len(sub["rel_l2_vs_fp64"]["fp32"]) else 0.0
        eb = sub["rel_l2_vs_fp64"]["bf16"][k] if sub and k < len(sub["rel_l2_vs_fp64"]["bf16"]) else 0.0
        within.append(e is not None and e + gap <= 1e-3 and eb <= 1e-3)
    kstar = next((k for k in range(len(within)) if within[k]), None)
    last = next((k for k in range(len(within)) if not within[k]), len(within))
    line["within_1e-3_at_iteration"] = within
    line["value"] = round(tk[kstar] / t_plain, 4) if kstar is not None else None
    line["first_iteration_within_1e-3"] = None if kstar is None else kstar + 1
    line["within_1e-3_through_iteration"] = last if kstar == 0 else None
    line["target"] = "< 10 plain FP32 migrations"
    print(json.dumps(line), flush=True)


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
    ap.add_argument("--image", type=int, default=NX,
                    help="survey workload: image columns per side (smaller only for profiling captures)")
    ap.add_argument("--survey-traces", type=int, default=SURVEY_TRACES,
                    help="traces synthesised on the device (smaller only for profiling captures)")
    ap.add_argument("--cpu-traces", type=int, default=3000)
    ap.add_argument("--ref-traces", type=int, default=1500)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cg-iters", type=int, default=20, help="lsm workload: CG iterations")
    ap.add_argument("--lsm-ref-iters", type=int, default=20,
                    help="lsm workload: iterations of the full-size FP32-stored reference CGLS (0: none)")
    ap.add_argument("--fd-dirs", type=int, default=16,
                    help="lsm workload: finite-difference checks of the misfit gradient (random directions)")
    ap.add_argument("--autotune", type=int, default=-1,
                    help="survey workload: autotune the launch on this many traces before timing (<= 0: default "
                         "launch); line workload: > 0 autotunes on the line, else the launch the autotuner picks there")
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
