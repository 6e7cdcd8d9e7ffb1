"""Generate the golden fixtures of the measured workloads from the reference itself.

Runs the reference's own solver classes (compiled from its sources into
oracle/_ref/ by oracle/Makefile; the checkout is named by the
SPARSESOLV_REFERENCE environment variable or the Makefile's default) on:

  * the 80^3 curl-curl system with three seeded iron blocks
    (sparsesolv_gb300.voxel.config2, n = 1,497,840): shifted ICCG at
    alpha 1.0 (capped at 300 iterations: the unshifted factor does not reach
    1e-8), 1.05, 1.1, 1.2 and 1.3, shifted IC-MRTR at 1.1, and the default
    Eisenstat SGS-MRTR;
  * the 60^3 complex eddy-current system (voxel.config3, n = 626,580):
    shifted IC-MRTR and COCG at alpha 1.1;
  * the reference's own sensitivity to rounding: the same solve with every
    entry of b moved by at most one unit in the last place (seeded), several
    times. The spread of its iteration counts (complex systems), and on the
    real 80^3 runs also of its residual log (per entry, relative to the
    unperturbed log) and of its solution (relative 2-norm), bounds what another
    rounding of the same arithmetic can be expected to give.

Writes tests/golden/golden_large.json (iteration counts, convergence, full
residual logs, the norm and 256 seeded samples of each solution, sha256 of
every input). The solution vectors themselves are too large to commit; the
GPU tests compare the full x with an FP64 oracle solve run in the test.

    python tests/golden/make_golden_large.py [--skip-sensitivity | --sensitivity-only]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle.oracle import Reference, Settings, build  # noqa: E402
from sparsesolv_gb300 import voxel  # noqa: E402

OUT = os.path.join(HERE, "golden_large.json")
N_SAMPLES = 256


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def sample_index(n):
    """The seeded solution entries stored per run (the same on every machine)."""
    return np.sort(np.random.default_rng(12345).choice(n, size=min(N_SAMPLES, n), replace=False))


def cases():
    return {"cfg2": voxel.config2(), "cfg3": voxel.config3()}


# (case, run name, method, settings, maxit)
RUNS = [
    ("cfg2", "iccg_a1.00", "iccg", Settings(accel_factor=1.0), 300),
    ("cfg2", "iccg_a1.05", "iccg", Settings(accel_factor=1.05), 5000),
    ("cfg2", "iccg_a1.10", "iccg", Settings(accel_factor=1.1), 5000),
    ("cfg2", "iccg_a1.20", "iccg", Settings(accel_factor=1.2), 5000),
    ("cfg2", "iccg_a1.30", "iccg", Settings(accel_factor=1.3), 5000),
    ("cfg2", "mrtr_ic_a1.10", "mrtr", Settings(accel_factor=1.1, precondition_type=0), 5000),
    ("cfg2", "mrtr_sgs", "mrtr", Settings(precondition_type=1), 5000),
    ("cfg3", "mrtr_ic_a1.10", "mrtr", Settings(accel_factor=1.1, precondition_type=0), 5000),
    ("cfg3", "iccg_a1.10", "iccg", Settings(accel_factor=1.1), 5000),
]
# (case, run) whose sensitivity to one-ulp changes of b is measured, and how many times
SENSITIVITY = [("cfg3", "mrtr_ic_a1.10", 6), ("cfg3", "iccg_a1.10", 6), ("ec8", "iccg", 16), ("ec8", "mrtr_ic", 16)]
SENSITIVITY += [("cfg2", run, 4) for _, run, _, _, _ in RUNS[:7]]


def ulp_perturbed(b, seed):
    """b with every entry moved by -1, 0 or +1 unit in the last place (real and
    imaginary parts independently), seeded."""
    rng = np.random.default_rng(seed)

    def move(v):
        s = rng.integers(-1, 2, size=v.shape)
        out = v.copy()
        up, dn = s > 0, s < 0
        out[up] = np.nextafter(v[up], np.inf)
        out[dn] = np.nextafter(v[dn], -np.inf)
        return out

    if np.iscomplexobj(b):
        return move(b.real) + 1j * move(b.imag)
    return move(b)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--skip-sensitivity", action="store_true")
    ap.add_argument("--sensitivity-only", action="store_true",
                    help="keep the committed runs, measure the sensitivity entries it lacks")
    args = ap.parse_args()
    build()
    ref = Reference()
    meta = {"cases": {}, "runs": {}, "sensitivity": {}, "samples": N_SAMPLES,
            "reference_threads": Reference.threads()}
    if os.path.exists(OUT) and (args.skip_sensitivity or args.sensitivity_only):
        with open(OUT) as f:
            old = json.load(f)
        meta["sensitivity"] = old.get("sensitivity", {})
        if args.sensitivity_only:
            meta = old
    systems = {}
    for name, case in cases().items():
        rp, ci, va, b = case.assemble()
        systems[name] = (rp, ci, va, b)
        meta["cases"][name] = {"n": int(len(rp) - 1), "nnz": int(len(ci)), "complex": bool(np.iscomplexobj(va)),
                               "sha256": digest(rp, ci, va, b)}
    for case, run, method, s, maxit in RUNS:
        if args.sensitivity_only:
            break
        rp, ci, va, b = systems[case]
        t0 = time.perf_counter()
        res = ref.solve(method, rp, ci, va, b, s, conv=1e-8, maxit=maxit)
        dt = time.perf_counter() - t0
        xs = res.x[sample_index(len(b))]
        meta["runs"][case + "/" + run] = {
            "method": method, "settings": s.__dict__, "maxit": maxit, "converged": bool(res.converged),
            "iters": int(len(res.log) - 1), "log": res.log.tolist(), "x_norm": float(np.linalg.norm(res.x)),
            "x_sample": ([[float(v.real), float(v.imag)] for v in xs] if np.iscomplexobj(xs)
                         else [float(v) for v in xs]),
            "seconds": dt}
        print(case, run, "iters", len(res.log) - 1, "converged", res.converged, "%.1f s" % dt, flush=True)
        with open(OUT, "w") as f:  # partial results survive an interrupted run
            json.dump(meta, f, indent=0, sort_keys=True)
    if not args.skip_sensitivity:
        sys.path.insert(0, HERE)
        import make_golden
        small = make_golden.cases()
        small_runs = {(c, r): (m, s) for c, r, m, s, _ in make_golden.RUNS}
        for case, run, reps in SENSITIVITY:
            if args.sensitivity_only and case + "/" + run in meta["sensitivity"]:
                continue
            if case in systems:
                rp, ci, va, b = systems[case]
                method, s, maxit = next((m, s, mx) for c, r, m, s, mx in RUNS if c == case and r == run)
            else:
                rp, ci, va, b = small[case]
                method, s = small_runs[(case, run)]
                maxit = 5000
            its = []
            real = not np.iscomplexobj(va) and case in systems
            if real:
                base = ref.solve(method, rp, ci, va, b, s, conv=1e-8, maxit=maxit)
                log_spread = np.zeros(len(base.log))
                x_spread = 0.0
            for k in range(reps):
                res = ref.solve(method, rp, ci, va, ulp_perturbed(b, 1000 + k), s, conv=1e-8, maxit=maxit)
                its.append(int(len(res.log) - 1))
                if real:
                    m = min(len(res.log), len(base.log))
                    d = np.abs(res.log[:m] - base.log[:m]) / np.abs(base.log[:m])
                    log_spread[:m] = np.maximum(log_spread[:m], d)
                    x_spread = max(x_spread, float(np.linalg.norm(res.x - base.x) / np.linalg.norm(base.x)))
            entry = {"perturbed_iters": its, "min": min(its), "max": max(its)}
            if real:
                entry["log_rel_spread"] = [float(v) for v in log_spread]
                entry["x_rel_spread"] = x_spread
            meta["sensitivity"][case + "/" + run] = entry
            print("sensitivity", case, run, its, flush=True)
            with open(OUT, "w") as f:
                json.dump(meta, f, indent=0, sort_keys=True)
    with open(OUT, "w") as f:
        json.dump(meta, f, indent=0, sort_keys=True)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
