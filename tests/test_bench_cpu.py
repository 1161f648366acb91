"""The benchmark's command-line contract, checked on a machine without a GPU.

* The reference arm (``--impl reference``: the oracle's FP32 transcription of the reference
  kernels on the host cores) prints one JSON line with the keys a reader of the benchmark
  parses: the metric and its unit, the step and warm-up counts, ``cpu_baseline`` describing the
  run and an ``e2e`` block whose value is the line's own with no host-device traffic.
* The GPU arm has no CPU path: without a CUDA device it exits non-zero and prints no line.
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


def test_gpu_arm_needs_a_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = run_bench("--workload", "c1", "--steps", "1", "--warmup", "3", "--no-cpu")
    assert p.returncode != 0
    assert not json_lines(p.stdout)
    assert "CUDA" in p.stderr
