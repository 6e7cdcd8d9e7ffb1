"""The C++ drop-in headers (include/SparseSolv/*.hpp) compile against the
C ABI library, and (on a GPU) the reference-style driver in
tests/cpp/dropin_example.cpp solves like the reference."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from sparsesolv_gb300 import _native, voxel

EXAMPLE = os.path.join(os.path.dirname(__file__), "cpp", "dropin_example.cpp")


def _compile(tmp_path):
    exe = str(tmp_path / "dropin")
    cmd = ["g++", "-std=c++17", "-O1", "-I", _native.INCLUDE, EXAMPLE, "-L", _native.PKG_DIR, "-lsparsesolv_gb300",
           "-Wl,-rpath," + _native.PKG_DIR, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_dropin_headers_compile_and_link(solver_lib, tmp_path):
    exe = _compile(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_dropin_example_solves(gpu, oracle, tmp_path):
    from oracle.oracle import Settings
    exe = _compile(tmp_path)
    rp, ci, va, b = voxel.curl_curl_case(10, seed=11).assemble()
    f = tmp_path / "sys.bin"
    with open(f, "wb") as fh:
        np.array([len(rp) - 1, len(ci)], np.int32).tofile(fh)
        rp.astype(np.int32).tofile(fh)
        ci.astype(np.int32).tofile(fh)
        va.astype(np.float64).tofile(fh)
        b.astype(np.float64).tofile(fh)
    out = subprocess.run([exe, str(f)], stdout=subprocess.PIPE, text=True, check=True).stdout.split()
    ok1, it1, ok2, it2 = int(out[0]), int(out[1]), int(out[2]), int(out[3])
    r1 = oracle.solve("iccg", rp, ci, va, b, Settings(accel_factor=1.1))
    r2 = oracle.solve("mrtr", rp, ci, va, b, Settings(precondition_type=1))
    assert ok1 and ok2 and it1 == r1.iters and it2 == r2.iters
    assert float(out[4]) == pytest.approx(r1.x[len(b) // 2], rel=1e-6, abs=1e-6 * np.abs(r1.x).max())
