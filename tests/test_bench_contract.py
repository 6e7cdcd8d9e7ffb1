"""The bench's command-line contract, on the CPU: defaults (one GPU, at least
three warm-up steps, the 80^3 workload) and the reference arm's JSON line for
the small 20^3 workload, which needs no GPU."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_defaults(monkeypatch):
    sys.path.insert(0, REPO)
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert a.gpus == 1 and a.warmup >= 3 and a.steps >= 1
    assert a.workload == "cfg2" and a.impl == "ours" and a.method == "iccg" and a.alpha == 1.1


def test_reference_arm_line():
    """Full solves on the host; the CUDA library of this package is never loaded."""
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'cfg1', '--steps', '1', "
            "'--warmup', '0', '--cpu-threads', '2']; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('CUDA_LIBRARY_LOADED' if 'libsparsesolv_gb300' in maps else 'CUDA_LIBRARY_NOT_LOADED')")
    out = subprocess.run([sys.executable, "-c", code],
                         cwd=REPO, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=600)
    assert "CUDA_LIBRARY_NOT_LOADED" in out.stdout, out.stdout[-2000:]
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "solves/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 1
    cb = d["cpu_baseline"]
    assert cb["cores"] == 2 and cb["kind"] in ("reference", "port") and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # a full solve to tolerance per step, with its phases, beside one on a single thread
    ph = d["phases"]
    assert ph["converged"] and ph["iterations"] == 30 and ph["true_relative_residual"] < 1e-8
    assert ph["setup_s"] > 0 and ph["per_iteration_s"] > 0 and abs(d["ms_per_step"] / 1e3 - ph["total_s"]) < 1.0
    assert d["one_thread"]["iterations"] == 30 and d["host"]["nproc"] >= 1
    # the workload named as the GPU arm names it
    import bench
    assert d["config"] == bench.workload_config(d["config"]["workload"], 21660, 658020, "shifted ICCG", "fp64", 1)
