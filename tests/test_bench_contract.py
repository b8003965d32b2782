"""The benchmark's JSON line: the keys and types its consumers read.

The reference arm (the oracle's restatement of the reference CPU path) runs here on the CPU; the engine's arm
needs a GPU and runs on a small slab with a short timed region.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*argv, timeout=900):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *argv], capture_output=True, text=True,
                         cwd=ROOT, timeout=timeout)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def check_common(b):
    for k, t in (("metric", str), ("value", float), ("unit", str), ("n_gpus", int), ("steps", int),
                 ("warmup", int), ("ms_per_step", float), ("higher_is_better", bool), ("scaling", str),
                 ("dtype", str), ("data", str), ("config", dict), ("cpu_baseline", dict), ("e2e", dict)):
        assert isinstance(b[k], t), (k, b.get(k))
    assert b["value"] > 0 and b["ms_per_step"] > 0
    assert b["vs_baseline"] is None
    assert b["config"]["workload"]
    e2e = b["e2e"]
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in e2e
    cpu = b["cpu_baseline"]
    for k in ("value", "unit", "cores", "kind", "sample"):
        assert k in cpu
    assert cpu["kind"] in ("port", "reference")


def test_reference_arm_line():
    b = run_bench("--impl", "reference", "--steps", "1", "--warmup", "0")
    check_common(b)
    assert b["impl"] == "reference"
    assert b["cpu_baseline"]["value"] == b["value"] and b["cpu_baseline"]["cores"] >= 1
    assert b["e2e"]["h2d_bytes_per_step"] == 0 and b["e2e"]["d2h_bytes_per_step"] == 0
    assert b["e2e"]["value"] == b["value"]


@pytest.mark.gpu
def test_engine_arm_line():
    b = run_bench("--n", "100000", "--steps", "20", "--warmup", "3", "--no-cpu-baseline", timeout=1200)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "dtype", "data", "config", "roofline", "e2e", "gpu_launches", "clocks"):
        assert k in b, k
    assert b["n_gpus"] == 1 and b["steps"] == 20 and b["warmup"] == 3
    assert b["value"] > 0 and b["gpu_launches"] > 0
    r = b["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert 0 < r["frac"] < 1.5 and r["achieved"] > 0
    e2e = b["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] == 24 * b["config"]["particles"]
    assert e2e["d2h_bytes_per_step"] >= 24 * b["config"]["particles"]
    assert b["force_error"]["pairs_equal"] and b["force_error"]["rms_rel"] < 1e-6
    assert "sm_mhz" in b["clocks"] and "reasons" in b["clocks"]
