"""The SparseMat drop-in's matrix API (include/SparseSolv/SparseMat.hpp) against
scipy on the same matrices, on the CPU: add (coefficient += with insertion),
compressed, isInclude, getTargetRowVal/ColVal, prune, printMat -> readMat
(real and complex), and with Eigen the triplet and Eigen-matrix constructors,
setMatrix and mat() (reference: include/SparseSolv/SparseMat.hpp:62-94,
src/SparseMat.cpp:54-409 of SparseSolv). The Eigen half compiles against the
Eigen copy vendored in the reference checkout and is skipped without it."""
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "cpp", "sparsemat_api.cpp")


def _run(tmp_path, eigen_dir=None):
    exe = str(tmp_path / ("api_eigen" if eigen_dir else "api"))
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"), SRC, "-o", exe]
    if eigen_dir:
        cmd[3:3] = ["-DWITH_EIGEN", "-I", eigen_dir]
    subprocess.run(cmd, check=True, capture_output=True)
    out = subprocess.run([exe, str(tmp_path)], check=True, capture_output=True, text=True).stdout
    return {ln.split()[0]: ln.split()[1:] for ln in out.splitlines()}


def _csr(fields):
    n, nnz = int(fields[0]), int(fields[1])
    rp = [int(v) for v in fields[2:3 + n]]
    ci = [int(v) for v in fields[3 + n:3 + n + nnz]]
    return rp, ci


def _eigen_dir():
    try:
        ref = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "print-ref"], check=True,
                             capture_output=True, text=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return None
    d = os.path.join(ref, "000_thirdparty")
    return d if os.path.exists(os.path.join(d, "Eigen", "Sparse")) else None


def test_sparsemat_api_without_eigen(tmp_path):
    r = _run(tmp_path)
    rows = [0, 0, 1, 1, 2, 3, 4, 0, 2]
    cols = [0, 1, 1, 3, 2, 3, 0, 0, 4]
    vals = [4.0, -1.0, 3.0, 0.5, 2.0, 1e-20, 7.0, 1.0, 1.5]
    A = sp.csr_matrix((vals, (rows, cols)), shape=(5, 5))
    A.sum_duplicates()
    assert _csr(r["coo"]) == (A.indptr.tolist(), A.indices.tolist())
    assert [float(v) for v in r["coo_val"]] == A.data.tolist()
    # add: (4, 4) and (4, 2) inserted in column order, (1, 1) accumulated
    A = A.tolil()
    A[4, 4] += 6.0
    A[1, 1] += 0.25
    A[4, 2] += -2.0
    A = A.tocsr()
    assert r["add_version"] == ["1"]
    assert _csr(r["add"]) == (A.indptr.tolist(), A.indices.tolist())
    assert [float(v) for v in r["add_val"]] == A.data.tolist()
    # isInclude: offset within the row, 0 when absent
    assert r["isInclude13"] == ["1", "1"] and r["isInclude20"] == ["0", "0"]
    col0 = A[:, 0].tocoo()
    exp = sorted(zip(col0.row.tolist(), col0.data.tolist()))
    got = r["col0"]
    assert [(int(got[i]), float(got[i + 1])) for i in range(0, len(got), 2)] == exp
    row4 = A[4].tocoo()
    got = r["row4"]
    assert [(int(got[i]), float(got[i + 1])) for i in range(0, len(got), 2)] == list(zip(row4.col.tolist(),
                                                                                       row4.data.tolist()))
    # printMat -> readMat: same pattern and values (%e text keeps 7 digits)
    assert _csr(r["read"]) == (A.indptr.tolist(), A.indices.tolist())
    assert np.allclose([float(v) for v in r["read_val"]], A.data, rtol=1e-6, atol=0)
    assert _csr(r["readc"]) == ([0, 1, 2, 3], [0, 2, 1])
    assert [float(v) for v in r["readc_val"]] == [1.5, -2.0, 0.0, 3.0, -4.0, 0.25]
    # prune(1.0) keeps |v| > 1e-12: the 1e-20 entry goes
    P = A.copy()
    P.data[np.abs(P.data) <= 1e-12] = 0
    P.eliminate_zeros()
    assert _csr(r["prune"]) == (P.indptr.tolist(), P.indices.tolist())


def test_sparsemat_eigen_interop(tmp_path):
    eig = _eigen_dir()
    if eig is None:
        pytest.skip("no Eigen checkout (the reference's vendored copy) on this machine")
    r = _run(tmp_path, eig)
    E = sp.csr_matrix(([4.0, 3.0, -1.0, -1.0, 1.0, 5.0, 0.5], ([0, 1, 0, 1, 0, 2, 2], [0, 1, 1, 0, 0, 2, 1])),
                      shape=(3, 3))
    E.sum_duplicates()
    assert _csr(r["trip"]) == (E.indptr.tolist(), E.indices.tolist())
    assert [float(v) for v in r["trip_val"]] == E.data.tolist()
    x = np.array([1.0, -2.0, 0.5])
    assert [float(v) for v in r["matvec"]] == (E @ x).tolist()
    assert r["lower_nnz"][0] == str(sp.tril(E).nnz) and float(r["lower_nnz"][2]) == E[1, 0]
    assert r["write"] == ["9", "version", "1"]
    M = sp.csr_matrix(([-1.0, 8.0, 2.0], ([0, 1, 1], [2, 0, 3])), shape=(2, 4))
    assert _csr(r["eigen"]) == (M.indptr.tolist(), M.indices.tolist())
    assert [float(v) for v in r["eigen_val"]] == M.data.tolist()
    assert r["eigen_cols"] == ["4"] and _csr(r["setmatrix"]) == (M.indptr.tolist(), M.indices.tolist())
    assert r["const_mat"] == ["2", "4", "3"]
