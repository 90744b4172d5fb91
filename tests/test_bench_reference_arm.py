"""The reference arm of bench.py, which runs beside the GPU arm: the compiled
reference kirchhoff() on the host cores over a bounded sample of the bench
survey, printed as one JSON line with the GPU arm's metric and unit, impl
"reference", a cpu_baseline describing the run and an e2e with no
host<->device bytes.  No GPU is involved."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_line():
    from oracle import refbuild
    try:
        refbuild.ensure_patched()
    except FileNotFoundError:
        pytest.skip("neither the reference sources nor their patched copy are here")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--ref-traces", "200"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "Gsample-trace pairs/s" and d["unit"] == "Gpairs/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1
    assert d["cpu_baseline"]["kind"] == "reference" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_roofline_constants_of_the_committed_profiles():
    """The ncu summaries that bench.py reads for its roofline sub-fields
    parse, and hold every figure it uses; whether they match the current
    kernel sources is reported per run in roofline.profile.stale."""
    sys.path.insert(0, str(ROOT))
    import bench
    for name in sorted(set(bench.PROFILE_OF.values())):
        pc = bench.profile_constants(name)
        assert pc is not None, name
        for key in ("kernel", "launch", "case", "source_sha256", "pairs", "warp_instructions", "issue_active",
                    "xu_pipe", "dram_bytes", "lts_bytes", "lts_throughput", "duration_ns", "image_columns"):
            assert key in pc, (name, key)
        assert set(pc["launch"]) >= {"tile_px", "samples_per_lane", "persistent", "ctas_per_sm"}, name
        assert pc["pairs"] > 0 and pc["warp_instructions"] > 0 and 0 < pc["issue_active"] <= 1, name
        assert len(pc["source_sha256"]) == len(bench.kernel_source_hash()), name
