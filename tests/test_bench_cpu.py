"""The benchmark's command-line contract and host logic, checked on a machine without a GPU.

* The reference arm (``--impl reference``: the oracle's FP32 transcription of the reference
  kernels on the host cores) prints one JSON line with the keys a reader of the benchmark
  parses: the metric and its unit, the step and warm-up counts, ``cpu_baseline`` describing the
  run and an ``e2e`` block whose value is the line's own with no host-device traffic.
* The GPU arm has no CPU path: without a CUDA device it exits non-zero and prints no line.
* The clocks record of the timed region is summarised from nvidia-smi samples as the timing
  rules read it (median SM clock, throttle reasons seen active).
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args):
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                          capture_output=True, text=True, timeout=600)


def json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def test_reference_arm_line():
    p = run_bench("--impl", "reference", "--workload", "c1", "--steps", "1", "--warmup", "3")
    assert p.returncode == 0, p.stderr[-2000:]
    lines = json_lines(p.stdout)
    assert len(lines) == 1, p.stdout[-2000:]
    d = lines[0]
    assert d["impl"] == "reference"
    for k in ("metric", "unit", "config"):
        assert d[k]
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] >= 3
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["higher_is_better"] is True
    assert d["config"]["workload"].startswith("c1")
    assert d["metric"].endswith("of one plain uniform SIRT iteration")   # C1's update rule
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_clock_summary_of_samples():
    """The clocks record of the timed region: median SM clock, the largest maximum clock and the
    throttle reasons seen active in any sample (nvidia-smi's csv, noheader, nounits form); no
    samples reads as unsampled."""
    sys.path.insert(0, ROOT)
    import bench

    s = bench.ClockSampler(0)                 # not entered: nothing runs nvidia-smi
    s.tmp.write("0, 2070, 2070, 900.50, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n"
                "0, 2055, 2070, 1391.2, 0x0000000000000004, Not Active, Not Active, Not Active, Active\n"
                "0, 2070, 2070, 1100.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n")
    d = s.summary()
    assert d == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    s = bench.ClockSampler(0)
    s.tmp.write("0, 1200, 2070, 700.0, 0x0000000000000040, Not Active, Active, Not Active, Not Active\n")
    assert s.summary()["reasons"] == ["hw_thermal_slowdown"]
    assert bench.ClockSampler(0).summary()["reasons"] == ["unsampled"]


def test_gpu_arm_needs_a_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = run_bench("--workload", "c1", "--steps", "1", "--warmup", "3", "--no-cpu")
    assert p.returncode != 0
    assert not json_lines(p.stdout)
    assert "CUDA" in p.stderr
