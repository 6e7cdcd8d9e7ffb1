"""Generate the golden fixtures from the reference itself.

Runs the reference's own solver classes, compiled from its sources into
oracle/_ref/ by oracle/Makefile (needs the SparseSolv checkout, named by the
SPARSESOLV_REFERENCE environment variable or the Makefile's default), on
seeded systems from sparsesolv_gb300.voxel and on the 5x5
example matrix of the reference's documentation (docs/html/Introduction.md of
SparseSolv). Writes tests/golden/golden.npz (residual logs, solutions, IC
factors) and tests/golden/golden.json (iteration counts, convergence flags,
sha256 of every input matrix so that generator drift is caught).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle.oracle import Reference, Settings, build  # noqa: E402
from sparsesolv_gb300 import voxel  # noqa: E402

DOC5 = np.array([
    [61.0, 0.0, 3.1, -0.1, 1.0],
    [0.0, 42.5, 2.0, 0.5, 4.0],
    [3.1, 2.0, 10.5, 0.0, 0.0],
    [-0.1, 0.5, 0.0, 80.4, 1.5],
    [1.0, 4.0, 0.0, 1.5, 1000.0],
])


def dense_to_csr(M):
    rp, ci, va = [0], [], []
    for i in range(M.shape[0]):
        for j in range(M.shape[1]):
            if abs(M[i, j]) > 1.0e-12:
                ci.append(j)
                va.append(M[i, j])
        rp.append(len(ci))
    return np.array(rp, np.int32), np.array(ci, np.int32), np.array(va)


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def cases():
    """name -> (row_ptr, col, val, b)"""
    out = {}
    rp, ci, va = dense_to_csr(DOC5)
    out["doc5"] = (rp, ci, va, np.arange(1.0, 6.0))
    c = voxel.curl_curl_case(10, seed=11)
    out["cc10"] = c.assemble()
    out["cfg1"] = voxel.config1().assemble()
    e = voxel.eddy_current_case(8, seed=7)
    out["ec8"] = e.assemble()
    out["cc6"] = voxel.curl_curl_case(6, seed=13, iron_size=2).assemble()
    out["ec5"] = voxel.eddy_current_case(5, seed=17).assemble()
    return out


# (case, run name, method, settings, store x)
RUNS = [
    ("doc5", "iccg", "iccg", Settings(accel_factor=1.0), True),
    ("cc10", "iccg", "iccg", Settings(accel_factor=1.1), True),
    ("cc10", "mrtr_ic", "mrtr", Settings(accel_factor=1.1, precondition_type=0), True),
    ("cc10", "mrtr_sgs", "mrtr", Settings(precondition_type=1), True),
    ("cc10", "iccg_diag", "iccg", Settings(accel_factor=1.1, is_diag_scale=True), True),
    ("cc10", "iccg_auto", "iccg", Settings(accel_factor=-1.0), False),
    ("cc10", "iccg_norm1", "iccg", Settings(accel_factor=1.1, conv_normalize_type=1), False),
    ("cfg1", "iccg", "iccg", Settings(accel_factor=1.1), False),
    ("cfg1", "mrtr_ic", "mrtr", Settings(accel_factor=1.1, precondition_type=0), False),
    ("cfg1", "mrtr_sgs", "mrtr", Settings(precondition_type=1), False),
    ("ec8", "iccg", "iccg", Settings(accel_factor=1.1), True),
    ("ec8", "mrtr_ic", "mrtr", Settings(accel_factor=1.1, precondition_type=0), True),
    ("ec8", "mrtr_sgs", "mrtr", Settings(precondition_type=1), False),
]
FACTORS = [("doc5", 1.0), ("doc5", 1.1), ("cc6", 1.1), ("ec5", 1.1)]


def main():
    build()
    ref = Reference()
    cs = cases()
    arrays, meta = {}, {"cases": {}, "runs": {}, "factors": {}}
    for name, (rp, ci, va, b) in cs.items():
        meta["cases"][name] = {"n": int(len(rp) - 1), "nnz": int(len(ci)), "complex": bool(np.iscomplexobj(va)),
                               "sha256": digest(rp, ci, va, b)}
    for case, run, method, s, keep_x in RUNS:
        rp, ci, va, b = cs[case]
        res = ref.solve(method, rp, ci, va, b, s, conv=1e-8, maxit=5000)
        key = case + "/" + run
        arrays[key + "/log"] = res.log
        if keep_x:
            arrays[key + "/x"] = res.x
        meta["runs"][key] = {"method": method, "converged": bool(res.converged), "iters": int(len(res.log) - 1),
                             "settings": s.__dict__}
    for case, alpha in FACTORS:
        rp, ci, va, b = cs[case]
        lrp, lci, lval, D = ref.ic_factor(rp, ci, va, alpha)
        key = "%s/ic%.2f" % (case, alpha)
        arrays[key + "/lrp"] = lrp
        arrays[key + "/lci"] = lci
        arrays[key + "/lval"] = lval
        arrays[key + "/D"] = D
        meta["factors"][key] = {"alpha": alpha}
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote", len(arrays), "arrays")


if __name__ == "__main__":
    main()
