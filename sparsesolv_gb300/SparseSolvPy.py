"""Drop-in for the reference's Python module ``SparseSolvPy``.

Same classes, method names, argument names and defaults as the reference's
pybind11 module (pybind/pybind.cpp:16-139 of SparseSolv):

    SparseBuilder(size)      getSize, initialize, reInitialize, add, resetMat
    SparseBuilderC(size)     get_size (sic), initialize, reInitialize, add, resetMat
    SparseMat()              SparseMat(builder, to_square=True)
                             SparseMat(n_nonzero, rows, cols, vals)
                             getSize, getMaxCol, print_mat(filename="Mat.csv")
    SparseMatC               the same for complex values
    MatSolverBase            setInitSolution, setDiagScale, setSaveBest, setSaveLog,
                             setDirvegeType (sic), setBadDivVal, setBadDivCount,
                             setConvNormalizeType, setConvNormalizeConst,
                             getResidualLog
    MatSolverICCG            setAccelFactor, solve_real, solve_complex
    MatSolverMRTR            setAccelFactor, setPreconditionType, solve_real, solve_complex

``solve_real(conv_cri, max_ite, A, b, x0)`` returns ``(converged, x)`` as the
reference does (x0 is copied; it is the initial guess only after
``setInitSolution(False)``). The solve itself runs on the GPU through the C
ABI; there is no CPU path. Additions beyond the reference: ``getIterations``,
``getTimings``, ``getAccelUsed``, ``setPrecision``, ``setReferenceQuirks``.
"""
from __future__ import annotations

import itertools

import numpy as np

from . import _capi

_token = itertools.count(1)


# ------------------------------------------------------------------ builders
class _BuilderBase:
    """Row-wise map accumulator: add() is +=, build() emits sorted triplets
    and empties the builder (src/SparseBuilder.cpp:107-141)."""

    _dtype = np.float64

    def __init__(self, size):
        self.initialize(size)

    def initialize(self, size):
        self._size = int(size)
        self._rows = [dict() for _ in range(self._size)]

    def reInitialize(self, size):
        self.initialize(size)

    def add(self, row, col, val):
        if row < 0 or row >= self._size or col < 0:
            raise IndexError("SparseBuilder.add: (%d, %d) outside %d rows" % (row, col, self._size))
        d = self._rows[row]
        d[col] = d.get(col, self._dtype(0)) + self._dtype(val)

    def resetMat(self):
        for d in self._rows:
            for k in d:
                d[k] = self._dtype(0)

    def _build(self, to_square):
        rows, cols, vals = [], [], []
        max_col = 0
        for i, d in enumerate(self._rows):
            for c in sorted(d):
                rows.append(i)
                cols.append(c)
                vals.append(d[c])
                max_col = max(max_col, c)
            self._rows[i] = dict()
        max_col += 1
        if to_square and max_col < self._size:
            rows.append(self._size - 1)
            cols.append(self._size - 1)
            vals.append(self._dtype(0))
            max_col = self._size
        return (np.asarray(rows, np.int64), np.asarray(cols, np.int64), np.asarray(vals, self._dtype),
                self._size, max_col)


class SparseBuilder(_BuilderBase):
    _dtype = np.float64

    def getSize(self):
        return self._size


class SparseBuilderC(_BuilderBase):
    _dtype = np.complex128

    def get_size(self):
        return self._size


# ------------------------------------------------------------------ matrices
class _MatBase:
    """Row-major CSR with sorted columns and summed duplicates (what
    Eigen::SparseMatrix<T, RowMajor>::setFromTriplets builds,
    src/SparseMat.cpp:80-122)."""

    _dtype = np.float64
    _builder = None

    def __init__(self, *args, **kw):
        self._token = next(_token)
        if not args and not kw:
            self._set(np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0, self._dtype), 0, 0)
            return
        if len(args) >= 1 and isinstance(args[0], _BuilderBase) or "builder" in kw:
            builder = kw.get("builder", args[0] if args else None)
            to_square = kw.get("to_square", args[1] if len(args) > 1 else True)
            if not isinstance(builder, self._builder):
                raise TypeError("builder type does not match the matrix type")
            r, c, v, nrows, ncols = builder._build(bool(to_square))
            self._from_coo(r, c, v, nrows, ncols)
            return
        names = ("n_nonzero", "rows", "cols", "vals")
        vals = dict(zip(names, args))
        vals.update(kw)
        nnz = int(vals["n_nonzero"])
        r = np.asarray(vals["rows"], np.int64)[:nnz]
        c = np.asarray(vals["cols"], np.int64)[:nnz]
        v = np.asarray(vals["vals"], self._dtype)[:nnz]
        nrows = int(r.max()) + 1 if nnz else 1
        ncols = int(c.max()) + 1 if nnz else 1
        self._from_coo(r, c, v, nrows, ncols)

    def _from_coo(self, r, c, v, nrows, ncols):
        if len(r) and (r.min() < 0 or c.min() < 0):
            raise IndexError("negative index")
        if nrows > np.iinfo(np.int32).max:
            raise OverflowError("SparseMat size exceeds slv_int range")
        key = r * max(ncols, 1) + c
        order = np.argsort(key, kind="stable")
        key_s = key[order]
        uniq, first = np.unique(key_s, return_index=True)
        vals = np.zeros(len(uniq), self._dtype)
        grp = np.repeat(np.arange(len(uniq)), np.diff(np.append(first, len(key_s))))
        np.add.at(vals, grp, v[order])
        rows_u = (uniq // max(ncols, 1)).astype(np.int64)
        cols_u = (uniq % max(ncols, 1)).astype(np.int32)
        rp = np.zeros(nrows + 1, np.int64)
        np.add.at(rp, rows_u + 1, 1)
        rp = np.cumsum(rp).astype(np.int32)
        self._set(rp, cols_u, vals, nrows, ncols)

    def _set(self, rp, ci, val, nrows, ncols):
        self.row_ptr = np.ascontiguousarray(rp, np.int32)
        self.col = np.ascontiguousarray(ci, np.int32)
        self.val = np.ascontiguousarray(val, self._dtype)
        self.shape = (int(nrows), int(ncols))

    @classmethod
    def from_csr(cls, row_ptr, col, val, ncols=None):
        """(addition) wrap an already sorted, duplicate-free CSR without copying semantics changes"""
        m = cls.__new__(cls)
        m._token = next(_token)
        n = len(row_ptr) - 1
        m._set(row_ptr, col, val, n, n if ncols is None else ncols)
        return m

    def getSize(self):
        return self.shape[0]

    def getMaxCol(self):
        return int(self.col.max()) if len(self.col) else 0

    def print_mat(self, filename="Mat.csv"):
        n = self.shape[0]
        with open(filename, "w") as fp:
            fp.write("Column size : %d\n" % n)
            for i in range(n):
                fp.write("%d\n" % (self.row_ptr[i + 1] - self.row_ptr[i]))
            fp.write("Column : \n")
            for i in range(n):
                a, b = self.row_ptr[i], self.row_ptr[i + 1]
                fp.write(("-1" if a == b else " ".join(str(c) for c in self.col[a:b]) + " ") + "\n")
            fp.write("Mat value : \n")
            for i in range(n):
                a, b = self.row_ptr[i], self.row_ptr[i + 1]
                fp.write("".join("%e " % x if not np.iscomplexobj(x) else "(%e,%e) " % (x.real, x.imag)
                                 for x in self.val[a:b]) + "\n")


class SparseMat(_MatBase):
    _dtype = np.float64
    _builder = SparseBuilder


class SparseMatC(_MatBase):
    _dtype = np.complex128
    _builder = SparseBuilderC


# ------------------------------------------------------------------ solvers
class MatSolverBase:
    """Settings and residual log of a solver (include/SparseSolv/MatSolverBase.hpp:124-137)."""

    _method = _capi.METHOD_ICCG

    def __init__(self):
        self._opt = _capi.Handle.default_options()
        self._h = None

    def _handle(self):
        if self._h is None:
            self._h = _capi.Handle(0)
        return self._h

    def setInitSolution(self, bl):
        self._opt.is_init = int(bool(bl))

    def setDiagScale(self, bl):
        self._opt.is_diag_scale = int(bool(bl))

    def setSaveBest(self, bl):
        self._opt.is_save_best = int(bool(bl))

    def setSaveLog(self, bl):
        self._opt.is_save_residual_log = int(bool(bl))

    def setDirvegeType(self, x):
        self._opt.diverge_judge_type = int(x)

    def setBadDivVal(self, x):
        self._opt.bad_div_val = float(x)

    def setBadDivCount(self, x):
        self._opt.bad_div_count_thres = int(x)

    def setConvNormalizeType(self, x):
        self._opt.conv_normalize_type = int(x)

    def setConvNormalizeConst(self, x):
        self._opt.conv_normalize_const = float(x)

    def getResidualLog(self):
        if self._h is None:
            return []
        return list(self._h.residual_log())

    # ---- additions
    def setPrecision(self, mode):
        """0 = FP64 throughout (default), 1 = FP32 inner loop with FP64 refinement."""
        self._opt.precision = int(mode)

    def setReferenceQuirks(self, bl):
        """Reproduce the reference's IC-MRTR p update and MRTR warm start."""
        self._opt.mrtr_reference_quirks = int(bool(bl))

    def getIterations(self):
        return 0 if self._h is None else self._h.iters()

    def getTimings(self):
        """(setup+factor ms, iterations ms) of the last solve."""
        return (0.0, 0.0) if self._h is None else tuple(self._h.timings())

    def getAccelUsed(self):
        return 0.0 if self._h is None else self._h.accel_used()

    def _solve(self, conv_cri, max_ite, A, b, x0, cplx, normB=-1.0):
        want = SparseMatC if cplx else SparseMat
        if not isinstance(A, want):
            raise TypeError("expected %s" % want.__name__)
        dt = np.complex128 if cplx else np.float64
        n = A.getSize()
        b = np.ascontiguousarray(b, dt).reshape(-1)
        x = np.array(x0, dt, copy=True).reshape(-1)
        if b.shape[0] != n or x.shape[0] != n:
            raise ValueError("vector sizes do not match the matrix (%d)" % n)
        h = self._handle()
        h.set_matrix(A.row_ptr, A.col, A.val, key=A._token)
        h.set_options(self._opt)
        ok = h.solve(self._method, b, x, conv=float(conv_cri), max_ite=int(max_ite), normB=float(normB))
        if not ok:
            print("not Convergence!!! ")
        return ok, x

    def solve_real(self, conv_cri, max_ite, A, b, x0):
        return self._solve(conv_cri, max_ite, A, b, x0, False)

    def solve_complex(self, conv_cri, max_ite, A, b, x0):
        return self._solve(conv_cri, max_ite, A, b, x0, True)


class MatSolverICCG(MatSolverBase):
    """Shifted ICCG (real) / ICCOCG (complex), default alpha 1.05."""

    _method = _capi.METHOD_ICCG

    def __init__(self):
        super().__init__()
        self._opt.accel_factor = 1.05

    def setAccelFactor(self, a):
        self._opt.accel_factor = float(a)


class MatSolverMRTR(MatSolverBase):
    """MRTR with IC (precondition type 0) or Eisenstat SGS (type 1, default)."""

    _method = _capi.METHOD_MRTR

    def __init__(self):
        super().__init__()
        self._opt.accel_factor = 1.05
        self._opt.precondition_type = 1

    def setAccelFactor(self, a):
        self._opt.accel_factor = float(a)

    def setPreconditionType(self, t):
        self._opt.precondition_type = int(t)
