"""bench.py's host logic on CPU: the algorithmic-byte count, the peak source,
the clock summary (throttle reasons from nvidia-smi rows), and the reference
arm's JSON line on the small Poisson workload (it runs the reference's CPU
loop, so it needs no GPU)."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def test_algorithmic_bytes_formula():
    import bench
    # nnz*(val+idx) + (rows+1)*ptr + rows*y + distinct*x
    assert bench.algorithmic_bytes(10, 100, 7, 4) == 100 * 8 + 11 * 4 + 10 * 4 + 7 * 4
    assert bench.algorithmic_bytes(8388608, 183752648, 8388608, 4) == 1570684484


def test_peaks_source(monkeypatch, tmp_path):
    import bench
    monkeypatch.setattr(bench, "ROOT", tmp_path)
    assert bench.peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6779.7}))
    assert bench.peaks() == (6779.7, "measured")


def test_clock_summary_reasons():
    import bench
    c = bench.ClockSampler(0)
    c.rows = [["0", "2070", "2070", "500.1", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"],
              ["0", "1980", "2070", "1390.0", "0x4", "Not Active", "Not Active", "Not Active", "Active"],
              ["0", "2070", "2070", "620.5", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"]]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"] and s["power_w_max"] == pytest.approx(1390.0)
    assert bench.ClockSampler(0).summary()["reasons"] == ["no samples"]


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "poisson16k",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == "spmv_effective_GBps" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["workload"] == "poisson16k" and line["config"]["nnz"] > 0
    # the same workload keys as the GPU arm's config (bench.workload_config), so both lines name one workload
    import bench
    want = bench.workload_config("poisson16k", 1, 1, 1, 1, 1, 1)
    assert set(line["config"]) == set(want)
    assert line["config"]["cols"] == 16384 and 0 < line["config"]["distinct_cols"] <= 16384
    assert line["config"]["parallelism"] == "replicas1" and "pinned bit-exact" in line["cpu_baseline"]["sample"]
