"""CPU-side checks of the boundary: the CUDA library builds for sm_103a,
loads, and exports every entry point the C header declares; the compiled
SparseSolvPy module (pybind11 bindings of the C++ drop-in classes) builds
matrices the way the reference's SparseBuilder / SparseMat do. No kernel is
launched here."""
import os
import re
import subprocess

import numpy as np
import pytest

from sparsesolv_gb300 import SparseSolvPy as ssp
from sparsesolv_gb300 import _capi, _native


def _declared():
    with open(os.path.join(_native.INCLUDE, "sparsesolv_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(ssg_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(solver_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _native.SOLVER_LIB], stdout=subprocess.PIPE,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (ssg_\w+)", out))
    declared = _declared()
    assert declared, "no declarations found"
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    assert sorted(declared) == sorted(_capi.EXPORTED)


def test_python_constants_match_the_header():
    """Every #define of the C header that the ctypes layer mirrors has the same value there."""
    with open(os.path.join(_native.INCLUDE, "sparsesolv_gb300.h")) as f:
        defines = dict(re.findall(r"#define\s+(SSG_\w+)\s+\(?(-?[0-9]+)", f.read()))
    pairs = {
        "SSG_OK": "SSG_OK", "SSG_NOT_CONVERGED": "SSG_NOT_CONVERGED", "SSG_ERR_ARG": "SSG_ERR_ARG",
        "SSG_ERR_CUDA": "SSG_ERR_CUDA", "SSG_ERR_NO_DIAGONAL": "SSG_ERR_NO_DIAGONAL",
        "SSG_ERR_TIMEOUT": "SSG_ERR_TIMEOUT", "SSG_ERR_NOMEM": "SSG_ERR_NOMEM", "SSG_ERR_STATE": "SSG_ERR_STATE",
        "SSG_METHOD_ICCG": "METHOD_ICCG", "SSG_METHOD_MRTR": "METHOD_MRTR", "SSG_REAL": "REAL",
        "SSG_COMPLEX": "COMPLEX", "SSG_PREC_FP64": "PREC_FP64", "SSG_PREC_MIXED": "PREC_MIXED",
    }
    for name, value in defines.items():
        if name.startswith("SSG_TUNE_"):
            pairs[name] = name[len("SSG_"):]
    tune = [n for n in defines if n.startswith("SSG_TUNE_")]
    assert len(tune) >= 10
    for c_name, py_name in pairs.items():
        assert c_name in defines, c_name
        assert getattr(_capi, py_name) == int(defines[c_name]), (c_name, py_name)
    # (1 << 21) is written as a shift in the header
    assert _capi.NOALLOC_MAX_ROWS == 1 << 21


def test_library_is_built_for_sm_103a(solver_lib):
    # the fatbinary names the target architecture in its ELF notes; cuobjdump is
    # not needed, the gencode is recorded by the build recipe
    assert "arch=compute_103a,code=sm_103a" in " ".join(_native.ARCH_FLAGS)
    assert os.path.getsize(_native.SOLVER_LIB) > 100_000


def test_default_options_match_reference(solver_lib):
    o = _capi.Handle.default_options()
    assert (o.is_init, o.is_diag_scale, o.is_save_best, o.is_save_residual_log) == (1, 0, 0, 0)
    assert (o.diverge_judge_type, o.bad_div_val, o.bad_div_count_thres) == (0, 1000.0, 1000)
    assert (o.conv_normalize_type, o.conv_normalize_const) == (0, 1.0)
    assert o.accel_factor == 1.05 and o.precondition_type == 1 and o.precision == 0


def test_builder_accumulates_and_squares():
    b = ssp.SparseBuilder(4)
    b.add(0, 0, 1.0)
    b.add(0, 0, 2.0)
    b.add(1, 2, 5.0)
    b.add(2, 1, 5.0)
    assert b.getSize() == 4
    A = ssp.SparseMat(b)  # pybind default to_square=True: pads (3,3) with a zero
    assert A.shape == (4, 4)
    assert A.row_ptr.tolist() == [0, 1, 2, 3, 4]
    assert A.col.tolist() == [0, 2, 1, 3] and A.val.tolist() == [3.0, 5.0, 5.0, 0.0]
    assert A.getMaxCol() == 3
    # building empties the builder (src/SparseBuilder.cpp:552-553)
    B = ssp.SparseMat(b, False)
    assert len(B.col) == 0


def test_builder_c_spelling_and_complex():
    b = ssp.SparseBuilderC(2)
    assert b.get_size() == 2
    b.add(0, 0, 1 + 1j)
    b.add(1, 1, 2.0)
    A = ssp.SparseMatC(b)
    assert A.val.dtype == np.complex128 and A.val.tolist() == [1 + 1j, 2 + 0j]


def test_coo_constructor_sums_duplicates_and_sizes():
    A = ssp.SparseMat(5, [0, 1, 1, 2, 0], [0, 1, 1, 2, 0], [1.0, 2.0, 3.0, 4.0, 5.0])
    assert A.getSize() == 3
    assert A.row_ptr.tolist() == [0, 1, 2, 3] and A.val.tolist() == [6.0, 5.0, 4.0]


def test_sparsesolvpy_is_the_compiled_module_over_the_cpp_classes():
    assert ssp.__file__ == _native.PYBIND_MOD and ssp.__file__.endswith(".so")
    for name in ("SparseBuilder", "SparseBuilderC", "SparseMat", "SparseMatC", "MatSolverBase", "MatSolverICCG",
                 "MatSolverMRTR"):
        assert type(getattr(ssp, name)).__name__ == "pybind11_type", name
    assert issubclass(ssp.MatSolverICCG, ssp.MatSolverBase) and issubclass(ssp.MatSolverMRTR, ssp.MatSolverBase)


def test_sparsesolvpy_argument_errors():
    with pytest.raises(IndexError):
        ssp.SparseMat(2, [0, -1], [0, 0], [1.0, 2.0])
    with pytest.raises(ValueError):
        ssp.SparseMat(3, [0, 1], [0, 1], [1.0, 2.0])
    b = ssp.SparseBuilder(2)
    with pytest.raises(IndexError):
        b.add(2, 0, 1.0)
    A = ssp.SparseMat(2, [0, 1], [0, 1], [1.0, 2.0])
    with pytest.raises(IndexError):
        A.add(0, 5, 1.0)
    with pytest.raises(ValueError):
        ssp.SparseMat.from_csr(np.array([0, 2, 1], np.int32), np.array([0, 1], np.int32), np.ones(2))
    with pytest.raises(ValueError):
        ssp.SparseMat.from_csr(np.array([0, 2, 2], np.int32), np.array([1, 0], np.int32), np.ones(2))


def test_sparsesolvpy_matrix_additions():
    b = ssp.SparseBuilder(3)
    b.addMany(np.array([0, 1, 2, 0]), np.array([0, 1, 2, 0]), np.array([1.0, 2.0, 3.0, 4.0]))
    A = ssp.SparseMat(b)
    assert A.val.tolist() == [5.0, 2.0, 3.0]
    A.add(0, 2, -1.0)
    assert A.row_ptr.tolist() == [0, 2, 3, 4] and A.col.tolist() == [0, 2, 1, 2]
    assert A.isInclude(0, 2) == (True, 1) and A.isInclude(1, 0) == (False, 0)
    assert A.getTargetRowVal(2) == ([0, 2], [-1.0, 3.0]) and A.getTargetColVal(0) == ([0, 2], [5.0, -1.0])
    A.add(1, 1, -2.0)
    A.prune(1.0)
    assert A.nonZeros() == 3 and A.col.tolist() == [0, 2, 2]
    B = ssp.SparseMat.from_csr(A.row_ptr, A.col, A.val)
    assert B.shape == (3, 3) and B.val.tolist() == A.val.tolist()


def test_print_mat(tmp_path):
    A = ssp.SparseMat(3, [0, 1, 1], [0, 0, 1], [1.0, 2.0, 3.0])
    p = tmp_path / "m.csv"
    A.print_mat(str(p))
    text = p.read_text().splitlines()
    assert text[0] == "Column size : 2" and text[1:3] == ["1", "2"] and text[3] == "Column : "


def test_solver_setters_without_gpu(solver_lib):
    s = ssp.MatSolverMRTR()
    s.setPreconditionType(0)
    s.setAccelFactor(1.2)
    s.setDiagScale(True)
    s.setSaveLog(True)
    s.setDirvegeType(1)
    o = s.options
    assert o["precondition_type"] == 0 and o["accel_factor"] == 1.2
    assert o["is_diag_scale"] == 1 and o["is_save_residual_log"] == 1 and o["diverge_judge_type"] == 1
    assert s.getResidualLog() == []
    # defaults of the reference: alpha 1.05, SGS for MRTR, IC for ICCG
    assert ssp.MatSolverMRTR().options["precondition_type"] == 1
    assert ssp.MatSolverICCG().options["accel_factor"] == 1.05


def test_no_cpu_fallback_when_library_missing(monkeypatch):
    monkeypatch.setattr(_native, "SOLVER_LIB", "/nonexistent/libsparsesolv_gb300.so")
    monkeypatch.setattr(_native, "_solver", None)
    with pytest.raises(RuntimeError, match="CUDA library"):
        _native.load_solver()
