"""ctypes front end of the CPU checkers (TEST INFRASTRUCTURE ONLY).

``Oracle`` wraps ``liboracle.so`` (the C restatement in sparsesolv_oracle.c);
``Reference`` wraps ``_ref/libsparsesolv_ref.so`` (the reference's own solver
sources compiled by oracle/Makefile), which exists only where the reference
checkout was available at build time. Only tests, ``__graft_entry__.smoke``
and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libsparsesolv_ref.so")


def build(force=False):
    """Build liboracle.so, and _ref/ when the reference checkout is present
    (oracle/Makefile's ref-if-present: the SPARSESOLV_REFERENCE environment
    variable names the checkout; without one the step prints a message)."""
    cmd = ["make", "-s", "-C", HERE, "all"]
    if force:
        cmd.insert(1, "-B")
    subprocess.run(cmd, check=True)
    subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref-if-present"], check=True,
                   stdout=subprocess.DEVNULL if os.path.exists(REF_LIB) else None)


class _Opts(ctypes.Structure):
    _fields_ = [("is_init", ctypes.c_int), ("is_diag_scale", ctypes.c_int), ("is_save_best", ctypes.c_int),
                ("is_save_residual_log", ctypes.c_int), ("diverge_judge_type", ctypes.c_int),
                ("bad_div_val", ctypes.c_double), ("bad_div_count_thres", ctypes.c_int),
                ("conv_normalize_type", ctypes.c_int), ("conv_normalize_const", ctypes.c_double),
                ("accel_factor", ctypes.c_double), ("precondition_type", ctypes.c_int),
                ("mrtr_reference_quirks", ctypes.c_int)]


@dataclass
class Settings:
    """Solver settings with the reference's defaults (MatSolverBase.cpp:32-47,
    MatSolverICCG.hpp:40, MatSolverMRTR.hpp:40-43); save_log on for tests."""
    is_init: bool = True
    is_diag_scale: bool = False
    is_save_best: bool = False
    is_save_residual_log: bool = True
    diverge_judge_type: int = 0
    bad_div_val: float = 1000.0
    bad_div_count_thres: int = 1000
    conv_normalize_type: int = 0
    conv_normalize_const: float = 1.0
    accel_factor: float = 1.05
    precondition_type: int = 1
    mrtr_reference_quirks: bool = False

    def c(self):
        return _Opts(int(self.is_init), int(self.is_diag_scale), int(self.is_save_best),
                     int(self.is_save_residual_log), int(self.diverge_judge_type), float(self.bad_div_val),
                     int(self.bad_div_count_thres), int(self.conv_normalize_type),
                     float(self.conv_normalize_const), float(self.accel_factor), int(self.precondition_type),
                     int(self.mrtr_reference_quirks))


@dataclass
class Result:
    converged: bool
    x: np.ndarray
    log: np.ndarray
    iters: int


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class _Base:
    lib = None

    def _solve(self, fn, opts_c, method, rp, ci, val, b, x0, normB, conv, maxit, extra_iters):
        n = len(rp) - 1
        cplx = np.iscomplexobj(val) or np.iscomplexobj(b)
        dt = np.complex128 if cplx else np.float64
        rp = np.ascontiguousarray(rp, np.int32)
        ci = np.ascontiguousarray(ci, np.int32)
        val = np.ascontiguousarray(val, dt)
        b = np.ascontiguousarray(b, dt)
        x = np.zeros(n, dt) if x0 is None else np.array(x0, dt, copy=True)
        cap = maxit + 2
        log = np.zeros(cap)
        log_len = ctypes.c_int(0)
        iters = ctypes.c_int(0)
        args = [ctypes.byref(opts_c), ctypes.c_int(method), ctypes.c_int(n), _p(rp), _p(ci), _p(val), _p(b),
                ctypes.c_double(-1.0 if normB is None else normB), ctypes.c_double(conv), ctypes.c_int(maxit),
                _p(x), _p(log), ctypes.c_int(cap), ctypes.byref(log_len)]
        if extra_iters:
            args.append(ctypes.byref(iters))
        rc = fn(*args)
        if rc < 0:
            raise RuntimeError("solver error %d" % rc)
        ll = log_len.value
        it = iters.value if extra_iters else max(ll - 1, 0)
        return Result(bool(rc), x, log[:min(ll, cap)].copy(), it)


class Oracle(_Base):
    """The C restatement of the reference's solvers."""

    def __init__(self):
        if not os.path.exists(ORACLE_LIB):
            build()
        self.lib = ctypes.CDLL(ORACLE_LIB)

    def threads(self):
        """Host threads of the row-parallel SpMV (1 when built without OpenMP)."""
        return int(self.lib.or_threads())

    def set_threads(self, k):
        """Threads of the row-parallel SpMV for the following solves."""
        self.lib.or_set_threads(ctypes.c_int(int(k)))

    def last_timings(self):
        """Seconds of the last solve: (set-up incl. the IC factor, iterations, total)."""
        t = np.zeros(3)
        self.lib.or_last_timings(_p(t))
        return float(t[0]), float(t[1]), float(t[2])

    def solve(self, method, rp, ci, val, b, settings=None, x0=None, normB=None, conv=1e-8, maxit=10000):
        """method: 'iccg' or 'mrtr' (settings.precondition_type picks IC=0 / SGS=1)."""
        s = settings or Settings()
        cplx = np.iscomplexobj(val) or np.iscomplexobj(b)
        fn = self.lib.or_solve_z if cplx else self.lib.or_solve_d
        fn.restype = ctypes.c_int
        return self._solve(fn, s.c(), 0 if method == "iccg" else 1, rp, ci, val, b, x0, normB, conv, maxit, True)

    def ic_factor(self, rp, ci, val, alpha):
        n = len(rp) - 1
        cplx = np.iscomplexobj(val)
        dt = np.complex128 if cplx else np.float64
        lrp = np.zeros(n + 1, np.int32)
        lci = np.zeros(len(ci), np.int32)
        lval = np.zeros(len(ci), dt)
        D = np.zeros(n, dt)
        rp = np.ascontiguousarray(rp, np.int32)
        ci = np.ascontiguousarray(ci, np.int32)
        val = np.ascontiguousarray(val, dt)
        fn = self.lib.or_ic_factor_z if cplx else self.lib.or_ic_factor_d
        rc = fn(ctypes.c_int(n), _p(rp), _p(ci), _p(val), ctypes.c_double(alpha), _p(lrp), _p(lci), _p(lval), _p(D))
        if rc == -2:
            raise RuntimeError("there is not diagonal element!")
        nl = lrp[n]
        return lrp, lci[:nl].copy(), lval[:nl].copy(), D

    def ic_apply(self, lrp, lci, lval, D, r):
        n = len(lrp) - 1
        cplx = np.iscomplexobj(lval)
        dt = np.complex128 if cplx else np.float64
        z = np.zeros(n, dt)
        r = np.ascontiguousarray(r, dt)
        fn = self.lib.or_ic_apply_z if cplx else self.lib.or_ic_apply_d
        fn(ctypes.c_int(n), _p(np.ascontiguousarray(lrp, np.int32)), _p(np.ascontiguousarray(lci, np.int32)),
           _p(np.ascontiguousarray(lval, dt)), _p(np.ascontiguousarray(D, dt)), _p(r), _p(z))
        return z

    def spmv(self, rp, ci, val, x):
        n = len(rp) - 1
        cplx = np.iscomplexobj(val) or np.iscomplexobj(x)
        dt = np.complex128 if cplx else np.float64
        y = np.zeros(n, dt)
        fn = self.lib.or_spmv_z if cplx else self.lib.or_spmv_d
        fn(ctypes.c_int(n), _p(np.ascontiguousarray(rp, np.int32)), _p(np.ascontiguousarray(ci, np.int32)),
           _p(np.ascontiguousarray(val, dt)), _p(np.ascontiguousarray(x, dt)), _p(y))
        return y

    def levels(self, rp, ci, lower=True):
        """(level[n], perm[n], lptr[nlev+1]) of the forward (lower) or backward sweep."""
        n = len(rp) - 1
        level = np.zeros(n, np.int32)
        perm = np.zeros(n, np.int32)
        lptr = np.zeros(n + 2, np.int32)
        rp = np.ascontiguousarray(rp, np.int32)
        ci = np.ascontiguousarray(ci, np.int32)
        nlev = self.lib.or_levels(ctypes.c_int(n), _p(rp), _p(ci), ctypes.c_int(1 if lower else 0),
                                  _p(level), _p(perm), _p(lptr))
        return level, perm, lptr[:nlev + 1].copy()

    def triangle(self, rp, ci, lower=True):
        n = len(rp) - 1
        trp = np.zeros(n + 1, np.int32)
        tci = np.zeros(len(ci), np.int32)
        src = np.zeros(len(ci), np.int32)
        self.lib.or_triangle_pattern(ctypes.c_int(n), _p(np.ascontiguousarray(rp, np.int32)),
                                     _p(np.ascontiguousarray(ci, np.int32)), ctypes.c_int(1 if lower else 0),
                                     _p(trp), _p(tci), _p(src))
        m = trp[n]
        return trp, tci[:m].copy(), src[:m].copy()

    def transpose(self, rp, ci):
        n = len(rp) - 1
        trp = np.zeros(n + 1, np.int32)
        tci = np.zeros(len(ci), np.int32)
        src = np.zeros(len(ci), np.int32)
        self.lib.or_transpose_pattern(ctypes.c_int(n), _p(np.ascontiguousarray(rp, np.int32)),
                                      _p(np.ascontiguousarray(ci, np.int32)), _p(trp), _p(tci), _p(src))
        return trp, tci, src


class Reference(_Base):
    """The reference's own solver classes compiled from its sources."""

    @staticmethod
    def available():
        return os.path.exists(REF_LIB)

    def __init__(self):
        if not os.path.exists(REF_LIB):
            raise RuntimeError("reference build %s is missing" % REF_LIB)
        self.lib = ctypes.CDLL(REF_LIB)

    @staticmethod
    def threads():
        """OpenMP threads of the reference build (its Eigen SpMV is row-parallel)."""
        return int(os.environ.get("OMP_NUM_THREADS") or os.cpu_count() or 1)

    def solve(self, method, rp, ci, val, b, settings=None, x0=None, normB=None, conv=1e-8, maxit=10000):
        s = settings or Settings()
        if s.mrtr_reference_quirks is False and method == "mrtr":
            pass  # the reference always has its own behaviour
        cplx = np.iscomplexobj(val) or np.iscomplexobj(b)
        fn = self.lib.ref_solve_z if cplx else self.lib.ref_solve_d
        fn.restype = ctypes.c_int
        return self._solve(fn, s.c(), 0 if method == "iccg" else 1, rp, ci, val, b, x0, normB, conv, maxit, False)

    def ic_factor(self, rp, ci, val, alpha):
        n = len(rp) - 1
        cplx = np.iscomplexobj(val)
        dt = np.complex128 if cplx else np.float64
        lrp = np.zeros(n + 1, np.int32)
        lci = np.zeros(len(ci), np.int32)
        lval = np.zeros(len(ci), dt)
        D = np.zeros(n, dt)
        fn = self.lib.ref_ic_factor_z if cplx else self.lib.ref_ic_factor_d
        fn(ctypes.c_int(n), _p(np.ascontiguousarray(rp, np.int32)), _p(np.ascontiguousarray(ci, np.int32)),
           _p(np.ascontiguousarray(val, dt)), ctypes.c_double(alpha), _p(lrp), _p(lci), _p(lval), _p(D))
        nl = lrp[n]
        return lrp, lci[:nl].copy(), lval[:nl].copy(), D

    def coo_to_csr(self, rows, cols, vals):
        """The reference's SparseMatTMPL COO constructor: (nrows, ncols, rp, ci, val)."""
        rows = np.ascontiguousarray(rows, np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        cplx = np.iscomplexobj(vals)
        dt = np.complex128 if cplx else np.float64
        v = np.ascontiguousarray(vals, dt)
        nnz = len(rows)
        nr, nc = ctypes.c_int(0), ctypes.c_int(0)
        rp = np.zeros(int(rows.max()) + 2 if nnz else 1, np.int32)
        ci = np.zeros(max(nnz, 1), np.int32)
        va = np.zeros(max(nnz, 1), dt)
        fn = self.lib.ref_coo_to_csr_z if cplx else self.lib.ref_coo_to_csr_d
        got = fn(ctypes.c_int(nnz), _p(rows), _p(cols), _p(v), ctypes.byref(nr), ctypes.byref(nc), _p(rp), _p(ci),
                 _p(va), ctypes.c_int(len(ci)))
        assert got >= 0
        return nr.value, nc.value, rp[:nr.value + 1].copy(), ci[:got].copy(), va[:got].copy()


def csr_from_coo(rows, cols, vals):
    """Restatement of SparseMatTMPL's COO constructor (src/SparseMat.cpp:80-104,
    which hands the triplets to Eigen's setFromTriplets): a matrix of
    (max row + 1) x (max col + 1), columns ascending within a row, duplicate
    (row, col) entries summed one after another in input order.
    Returns (nrows, ncols, row_ptr, col, val)."""
    rows = np.asarray(rows, np.int64)
    cols = np.asarray(cols, np.int64)
    vals = np.asarray(vals)
    if len(rows) == 0:
        return 0, 0, np.zeros(1, np.int32), np.zeros(0, np.int32), vals[:0].copy()
    nrows, ncols = int(rows.max()) + 1, int(cols.max()) + 1
    order = np.lexsort((cols, rows))  # stable: equal keys keep input order
    key = rows[order] * ncols + cols[order]
    head = np.ones(len(key), bool)
    head[1:] = key[1:] != key[:-1]
    start = np.flatnonzero(head)
    length = np.diff(np.append(start, len(key)))
    out = vals[order[start]].copy()
    for k in range(1, int(length.max())):  # sequential sums, entry k of every run at once
        m = length > k
        out[m] = out[m] + vals[order[start[m] + k]]
    r = rows[order[start]]
    rp = np.zeros(nrows + 1, np.int32)
    np.cumsum(np.bincount(r, minlength=nrows), out=rp[1:])
    return nrows, ncols, rp, cols[order[start]].astype(np.int32), out


# the local edge tables of Element::calcB (examples/VoxelFEM/Element.cpp:141-143)
_RK = (0, 0, 0, 0, 1, 1, -1, -1, 1, -1, -1, 1)
_SK = (1, -1, -1, 1, 0, 0, 0, 0, 1, 1, -1, -1)
_TK = (1, 1, -1, -1, 1, -1, -1, 1, 0, 0, 0, 0)


def flux_density(nx, ny, nz, h, ex, ey, ez, A):
    """Restatement of Element::calcB / calcRot (examples/VoxelFEM/Element.cpp:116-168)
    at every element centre (pos_rst = 0) of a uniform voxel grid: for the 12
    edges in the example's order, rot = sign * 1.0 / 8.0 / L_a / L_b (L = h / 2),
    B += A_edge * rot edge by edge, edges without an unknown skipped.
    Returns B[ne, 3], element index x + nx (y + ny z)."""
    A = np.asarray(A)
    L = h / 2.0
    zz, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x, y, z = xx.ravel(), yy.ravel(), zz.ravel()
    parts = [A.real, A.imag] if np.iscomplexobj(A) else [A]
    out = [np.zeros((x.size, 3)) for _ in parts]
    for i in range(12):
        r, s, t = float(_RK[i]), float(_SK[i]), float(_TK[i])
        cx, cy, cz = x.copy(), y.copy(), z.copy()
        if i < 4:
            cy += s > 0
            cz += t > 0
            m = ex
            rot = (0.0, t * 1.0 / 8.0 / L / L, -s * 1.0 / 8.0 / L / L)
        elif i < 8:
            cx += r > 0
            cz += t > 0
            m = ey
            rot = (-t * 1.0 / 8.0 / L / L, 0.0, r * 1.0 / 8.0 / L / L)
        else:
            cx += r > 0
            cy += s > 0
            m = ez
            rot = (s * 1.0 / 8.0 / L / L, -r * 1.0 / 8.0 / L / L, 0.0)
        ids = m[cx + (nx + 1) * (cy + (ny + 1) * cz)]
        ok = ids >= 0
        for p, o in zip(parts, out):
            a = p[ids[ok]]
            for c in range(3):
                o[ok, c] = o[ok, c] + a * rot[c]
    return out[0] + 1j * out[1] if len(out) == 2 else out[0]
