"""The bench line on a GPU, on the small cfg1 workload (21,660 unknowns): one JSON
line with the contract's keys (metric, value, unit, steps, warmup, ms_per_step,
e2e with its host/device byte counts and per-step times, gpu_launches, roofline,
cpu_baseline, clocks), positive rates, a converged solve at oracle parity, and a
roofline fraction computed from its own achieved and peak."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_line_on_cfg1(gpu):
    cmd = [sys.executable, os.path.join(REPO, "bench.py"), "--workload", "cfg1", "--steps", "3", "--warmup", "3",
           "--no-serving", "--no-batch"]
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "roofline", "cpu_baseline", "clocks"):
        assert key in d, key
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["gpu_launches"] > 0
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert 0 < e2e["step_ms"]["min"] <= e2e["step_ms"]["median"] <= e2e["step_ms"]["max"]
    rf = d["roofline"]
    assert rf["bound"] in ("hbm", "tensor") and rf["achieved"] > 0 and rf["peak"] > 0
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) <= 1e-9 * max(1.0, rf["frac"])
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
    assert d["parity"]["A_dx_over_b"] < 1e-6 and d["parity"]["gpu_iterations"] > 0
