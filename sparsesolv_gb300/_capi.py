"""ctypes declarations of the C ABI (include/sparsesolv_gb300.h) and a thin
handle class used by the Python mirror of the reference's module."""
from __future__ import annotations

import ctypes

import numpy as np

SSG_OK = 0
SSG_NOT_CONVERGED = 1
SSG_ERR_ARG = -1
SSG_ERR_CUDA = -2
SSG_ERR_NO_DIAGONAL = -3
SSG_ERR_TIMEOUT = -4
SSG_ERR_NOMEM = -5
SSG_ERR_STATE = -6
METHOD_ICCG = 0
METHOD_MRTR = 1
REAL = 0
COMPLEX = 1
PREC_FP64 = 0
PREC_MIXED = 1

EXPORTED = [
    "ssg_default_options", "ssg_create", "ssg_destroy", "ssg_last_error", "ssg_set_options", "ssg_set_matrix",
    "ssg_set_matrix_device", "ssg_set_matrix_coo", "ssg_get_matrix", "ssg_flux_density", "ssg_set_matrix_voxel", "ssg_solve", "ssg_solve_device", "ssg_solve_multi", "ssg_solve_multi_device", "ssg_get_residual_log", "ssg_get_iters",
    "ssg_get_accel_used", "ssg_get_timings", "ssg_factor", "ssg_apply_precond", "ssg_spmv", "ssg_level_schedule",
    "ssg_update_values", "ssg_update_values_device", "ssg_get_stream", "ssg_set_profiling", "ssg_get_kernel_stats",
    "ssg_launch_count", "ssg_set_tuning", "ssg_autotune", "ssg_ic_factor_noalloc", "ssg_batch_create", "ssg_batch_destroy",
    "ssg_batch_last_error", "ssg_batch_add", "ssg_batch_set_rhs", "ssg_batch_clear", "ssg_batch_start", "ssg_batch_poll", "ssg_batch_wait", "ssg_batch_step", "ssg_batch_finished",
    "ssg_batch_result", "ssg_batch_residual_log", "ssg_batch_timings", "ssg_batch_stream",
    "ssg_batch_set_profiling", "ssg_batch_kernel_stats", "ssg_batch_set_graphs", "ssg_batch_set_persistent", "ssg_batch_autotune", "ssg_batch_set_precision",
]
NOALLOC_MAX_ROWS = 1 << 21
TUNE_SWEEP_CTA_PER_SM = 0
TUNE_SWEEP_GROUP = 1
TUNE_SWEEP_BACKOFF_NS = 2
TUNE_FACTOR_BACKOFF_NS = 3
TUNE_RECIPROCAL_DIAG = 4
TUNE_SWEEP_MODE = 5
TUNE_CLUSTER_RING_KB = 6
TUNE_CLUSTER_GROUP = 7
TUNE_BATCH_GROUP = 8
TUNE_SPMV_GROUP = 9
TUNE_SPIN_LIMIT_US = 10
KERNEL_CLASSES = ["forward sweep", "backward sweep", "spmv", "vector", "ic factor", "level schedule"]


class Options(ctypes.Structure):
    _fields_ = [("is_init", ctypes.c_int), ("is_diag_scale", ctypes.c_int), ("is_save_best", ctypes.c_int),
                ("is_save_residual_log", ctypes.c_int), ("diverge_judge_type", ctypes.c_int),
                ("bad_div_val", ctypes.c_double), ("bad_div_count_thres", ctypes.c_int),
                ("conv_normalize_type", ctypes.c_int), ("conv_normalize_const", ctypes.c_double),
                ("accel_factor", ctypes.c_double), ("precondition_type", ctypes.c_int),
                ("precision", ctypes.c_int), ("mrtr_reference_quirks", ctypes.c_int)]


def declare(lib):
    H = ctypes.c_void_p
    P = ctypes.c_void_p
    I = ctypes.c_int
    D = ctypes.c_double
    pI = ctypes.POINTER(ctypes.c_int)
    sig = {
        "ssg_default_options": ([ctypes.POINTER(Options)], None),
        "ssg_create": ([ctypes.POINTER(ctypes.c_void_p), I], I),
        "ssg_destroy": ([H], I),
        "ssg_last_error": ([H], ctypes.c_char_p),
        "ssg_set_options": ([H, ctypes.POINTER(Options)], I),
        "ssg_set_matrix": ([H, I, I, P, P, P, I], I),
        "ssg_set_matrix_device": ([H, I, I, P, P, P, I], I),
        "ssg_set_matrix_coo": ([H, I, I, P, P, P, I, I], I),
        "ssg_get_matrix": ([H, P, P, P, pI, pI], I),
        "ssg_flux_density": ([H, I, I, I, D, D, D, P, P, P, I, P, I, P, I], I),
        "ssg_set_matrix_voxel": ([H, I, I, I, P, P, P, I, P, P, P, P, P, D, P, I, P, I], I),
        "ssg_solve": ([H, I, D, I, D, P, P], I),
        "ssg_solve_device": ([H, I, D, I, D, P, P], I),
        "ssg_solve_multi": ([H, I, D, I, I, P, P, P, P], I),
        "ssg_solve_multi_device": ([H, I, D, I, I, P, P, P, P], I),
        "ssg_get_residual_log": ([H, P, I, pI], I),
        "ssg_get_iters": ([H, pI], I),
        "ssg_get_accel_used": ([H, ctypes.POINTER(ctypes.c_double)], I),
        "ssg_get_timings": ([H, P, I], I),
        "ssg_factor": ([H, D, P, P, P, P, pI], I),
        "ssg_apply_precond": ([H, P, P], I),
        "ssg_spmv": ([H, P, P], I),
        "ssg_level_schedule": ([H, I, P, P, pI], I),
        "ssg_update_values": ([H, P], I),
        "ssg_update_values_device": ([H, P], I),
        "ssg_get_stream": ([H, ctypes.POINTER(ctypes.c_void_p)], I),
        "ssg_set_profiling": ([H, I], I),
        "ssg_get_kernel_stats": ([H, P, P, P, I], I),
        "ssg_launch_count": ([], ctypes.c_longlong),
        "ssg_set_tuning": ([H, I, I], I),
        "ssg_autotune": ([H, I, pI, pI, pI, ctypes.POINTER(ctypes.c_double)], I),
        "ssg_ic_factor_noalloc": ([I, I, P, P, P, P, P, D, I, P], I),
        "ssg_batch_create": ([ctypes.POINTER(ctypes.c_void_p), I], I),
        "ssg_batch_destroy": ([H], I),
        "ssg_batch_last_error": ([H], ctypes.c_char_p),
        "ssg_batch_add": ([H, I, I, P, P, P, I, I, P, pI], I),
        "ssg_batch_set_rhs": ([H, I, P], I),
        "ssg_batch_clear": ([H], I),
        "ssg_batch_start": ([H, I, D, D, I], I),
        "ssg_batch_poll": ([H, pI], I),
        "ssg_batch_wait": ([H], I),
        "ssg_batch_step": ([H, pI], I),
        "ssg_batch_finished": ([H, I, pI], I),
        "ssg_batch_result": ([H, I, P, P, P], I),
        "ssg_batch_residual_log": ([H, I, I, P, I, pI], I),
        "ssg_batch_timings": ([H, P], I),
        "ssg_batch_stream": ([H, ctypes.POINTER(ctypes.c_void_p)], I),
        "ssg_batch_set_profiling": ([H, I], I),
        "ssg_batch_set_graphs": ([H, I], I),
        "ssg_batch_set_persistent": ([H, I], I),
        "ssg_batch_autotune": ([H, P, P, P, P], I),
        "ssg_batch_set_precision": ([H, I, D], I),
        "ssg_batch_kernel_stats": ([H, P, P, P, I], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res


class SolverError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class Handle:
    """One device handle: a CUDA stream plus all device state of a solver."""

    def __init__(self, device=0):
        from ._native import load_solver
        self.lib = load_solver()
        h = ctypes.c_void_p()
        rc = self.lib.ssg_create(ctypes.byref(h), int(device))
        if rc != SSG_OK:
            raise SolverError(rc, "ssg_create failed")
        self.h = h
        self.n = 0
        self.complex = False
        self._mat_key = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.ssg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc < 0:
            msg = self.lib.ssg_last_error(self.h)
            raise SolverError(rc, "%s: %s" % (what, msg.decode() if msg else ""))
        return rc

    @staticmethod
    def default_options():
        from ._native import load_solver
        o = Options()
        load_solver().ssg_default_options(ctypes.byref(o))
        return o

    def set_options(self, o):
        self._check(self.lib.ssg_set_options(self.h, ctypes.byref(o)), "ssg_set_options")

    def set_matrix(self, row_ptr, col, val, key=None):
        """Upload a CSR matrix (numpy, host). ``key`` skips re-uploads of the same matrix."""
        if key is not None and key == self._mat_key:
            return
        rp = np.ascontiguousarray(row_ptr, np.int32)
        ci = np.ascontiguousarray(col, np.int32)
        cplx = np.iscomplexobj(val)
        v = np.ascontiguousarray(val, np.complex128 if cplx else np.float64)
        n = len(rp) - 1
        self._check(self.lib.ssg_set_matrix(self.h, n, len(ci), _p(rp), _p(ci), _p(v), COMPLEX if cplx else REAL),
                    "ssg_set_matrix")
        self.n = n
        self.complex = cplx
        self._mat_key = key

    def set_matrix_device(self, n, nnz, rp_ptr, ci_ptr, val_ptr, cplx):
        self._check(self.lib.ssg_set_matrix_device(self.h, n, nnz, ctypes.c_void_p(rp_ptr), ctypes.c_void_p(ci_ptr),
                                                   ctypes.c_void_p(val_ptr), COMPLEX if cplx else REAL),
                    "ssg_set_matrix_device")
        self.n = n
        self.complex = cplx
        self._mat_key = None

    def set_matrix_coo(self, n, rows, cols, vals):
        """n x n matrix from COO triplets (host numpy), built on the device; a
        repeated (row, col) is summed in input order."""
        r = np.ascontiguousarray(rows, np.int32)
        c = np.ascontiguousarray(cols, np.int32)
        cplx = np.iscomplexobj(vals)
        v = np.ascontiguousarray(vals, np.complex128 if cplx else np.float64)
        assert len(r) == len(c) == len(v)
        self._check(self.lib.ssg_set_matrix_coo(self.h, int(n), len(r), _p(r), _p(c), _p(v),
                                                COMPLEX if cplx else REAL, 0), "ssg_set_matrix_coo")
        self.n = int(n)
        self.complex = cplx
        self._mat_key = None

    def flux_density(self, case, A):
        """B = curl A at every voxel centre of a voxel case (sparsesolv_gb300.voxel),
        shape (nz, ny, nx, 3), from the solution A of its system."""
        ex, ey, ez = case.edge_maps()
        cplx = np.iscomplexobj(A)
        a = np.ascontiguousarray(A, np.complex128 if cplx else np.float64)
        B = np.zeros(case.nx * case.ny * case.nz * 3, a.dtype)
        h = case.h
        self._check(self.lib.ssg_flux_density(self.h, case.nx, case.ny, case.nz, float(h), float(h), float(h),
                                              _p(ex), _p(ey), _p(ez), len(a), _p(a), COMPLEX if cplx else REAL,
                                              _p(B), 0), "ssg_flux_density")
        return B.reshape(case.nz, case.ny, case.nx, 3)

    def set_matrix_voxel(self, case, complex_values=None, coils=None):
        """Assemble a voxel case's system (sparsesolv_gb300.voxel) on the device into this
        handle (ssg_set_matrix_voxel); returns its right-hand side b. Bit-identical to
        case.assemble()."""
        from . import voxel
        if complex_values is None:
            complex_values = case.sigma != 0.0 and case.omega != 0.0 and bool(case.conductors)
        ex, ey, ez = case.edge_maps()
        n = int(max(ex.max(), ey.max(), ez.max()) + 1)
        K, M, C = voxel.element_matrices(case.h)
        nu = case.nu()
        sig = case.sig() if complex_values else None
        tz = np.ascontiguousarray(case.tz(coils), np.float64)
        b = np.zeros(n, np.complex128 if complex_values else np.float64)
        self._check(self.lib.ssg_set_matrix_voxel(self.h, case.nx, case.ny, case.nz, _p(ex), _p(ey), _p(ez), n,
                                                  _p(K), _p(M), _p(C), _p(nu), _p(sig), float(case.omega), _p(tz),
                                                  COMPLEX if complex_values else REAL, _p(b), 0),
                    "ssg_set_matrix_voxel")
        self.n = n
        self.complex = bool(complex_values)
        self._mat_key = None
        return b

    def get_matrix(self):
        """(row_ptr, col, val) of the current matrix."""
        n, nnz = ctypes.c_int(0), ctypes.c_int(0)
        self._check(self.lib.ssg_get_matrix(self.h, None, None, None, ctypes.byref(n), ctypes.byref(nnz)),
                    "ssg_get_matrix")
        rp = np.zeros(n.value + 1, np.int32)
        ci = np.zeros(max(nnz.value, 1), np.int32)
        va = np.zeros(max(nnz.value, 1), np.complex128 if self.complex else np.float64)
        self._check(self.lib.ssg_get_matrix(self.h, _p(rp), _p(ci), _p(va), ctypes.byref(n), ctypes.byref(nnz)),
                    "ssg_get_matrix")
        return rp, ci[:nnz.value], va[:nnz.value]

    def solve(self, method, b, x, conv=1e-8, max_ite=10000, normB=-1.0):
        """Host arrays; x is updated in place. Returns True when converged."""
        dt = np.complex128 if self.complex else np.float64
        assert b.dtype == dt and x.dtype == dt and b.flags.c_contiguous and x.flags.c_contiguous
        rc = self._check(self.lib.ssg_solve(self.h, method, float(conv), int(max_ite), float(normB), _p(b), _p(x)),
                         "ssg_solve")
        return rc == SSG_OK

    def solve_multi(self, method, B, X, conv=1e-8, max_ite=10000):
        """B, X: host arrays (n_rhs, n); X is updated in place. Returns
        (all converged, iterations per right-hand side, status per right-hand side)."""
        dt = np.complex128 if self.complex else np.float64
        assert B.dtype == dt and X.dtype == dt and B.flags.c_contiguous and X.flags.c_contiguous
        assert B.ndim == 2 and B.shape == X.shape
        k = B.shape[0]
        it = np.zeros(k, np.int32)
        st = np.zeros(k, np.int32)
        rc = self._check(self.lib.ssg_solve_multi(self.h, method, float(conv), int(max_ite), k, _p(B), _p(X), _p(it),
                                                  _p(st)), "ssg_solve_multi")
        return rc == SSG_OK, it, st

    def solve_multi_device(self, method, nrhs, B_ptr, X_ptr, conv=1e-8, max_ite=10000):
        """Device pointers to nrhs vectors of n values each; returns
        (all converged, iterations per right-hand side, status per right-hand side)."""
        it = np.zeros(nrhs, np.int32)
        st = np.zeros(nrhs, np.int32)
        rc = self._check(self.lib.ssg_solve_multi_device(self.h, method, float(conv), int(max_ite), int(nrhs),
                                                         ctypes.c_void_p(B_ptr), ctypes.c_void_p(X_ptr), _p(it),
                                                         _p(st)), "ssg_solve_multi_device")
        return rc == SSG_OK, it, st

    def solve_device(self, method, b_ptr, x_ptr, conv=1e-8, max_ite=10000, normB=-1.0):
        rc = self._check(self.lib.ssg_solve_device(self.h, method, float(conv), int(max_ite), float(normB),
                                                   ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr)), "ssg_solve_device")
        return rc == SSG_OK

    def residual_log(self):
        n = ctypes.c_int(0)
        self._check(self.lib.ssg_get_residual_log(self.h, None, 0, ctypes.byref(n)), "ssg_get_residual_log")
        out = np.zeros(n.value)
        self._check(self.lib.ssg_get_residual_log(self.h, _p(out), n.value, ctypes.byref(n)), "ssg_get_residual_log")
        return out

    def iters(self):
        it = ctypes.c_int(0)
        self._check(self.lib.ssg_get_iters(self.h, ctypes.byref(it)), "ssg_get_iters")
        return it.value

    def accel_used(self):
        a = ctypes.c_double(0)
        self._check(self.lib.ssg_get_accel_used(self.h, ctypes.byref(a)), "ssg_get_accel_used")
        return a.value

    def timings(self):
        t = np.zeros(2)
        self._check(self.lib.ssg_get_timings(self.h, _p(t), 2), "ssg_get_timings")
        return t

    def factor(self, alpha):
        dt = np.complex128 if self.complex else np.float64
        n = self.n
        nnzL = ctypes.c_int(0)
        self._check(self.lib.ssg_factor(self.h, float(alpha), None, None, None, None, ctypes.byref(nnzL)), "ssg_factor")
        lrp = np.zeros(n + 1, np.int32)
        lci = np.zeros(max(nnzL.value, 1), np.int32)
        lval = np.zeros(max(nnzL.value, 1), dt)
        D = np.zeros(max(n, 1), dt)
        self._check(self.lib.ssg_factor(self.h, float(alpha), _p(lrp), _p(lci), _p(lval), _p(D), ctypes.byref(nnzL)),
                    "ssg_factor")
        return lrp, lci[:nnzL.value], lval[:nnzL.value], D[:n]

    def apply_precond(self, r):
        dt = np.complex128 if self.complex else np.float64
        r = np.ascontiguousarray(r, dt)
        z = np.zeros(self.n, dt)
        self._check(self.lib.ssg_apply_precond(self.h, _p(r), _p(z)), "ssg_apply_precond")
        return z

    def spmv(self, x):
        dt = np.complex128 if self.complex else np.float64
        x = np.ascontiguousarray(x, dt)
        y = np.zeros(self.n, dt)
        self._check(self.lib.ssg_spmv(self.h, _p(x), _p(y)), "ssg_spmv")
        return y

    def update_values(self, val):
        cplx = np.iscomplexobj(val)
        v = np.ascontiguousarray(val, np.complex128 if cplx else np.float64)
        self._check(self.lib.ssg_update_values(self.h, _p(v)), "ssg_update_values")

    def update_values_device(self, ptr):
        self._check(self.lib.ssg_update_values_device(self.h, ctypes.c_void_p(ptr)), "ssg_update_values_device")

    def stream(self):
        s = ctypes.c_void_p()
        self._check(self.lib.ssg_get_stream(self.h, ctypes.byref(s)), "ssg_get_stream")
        return s.value or 0

    def set_profiling(self, on):
        self._check(self.lib.ssg_set_profiling(self.h, 1 if on else 0), "ssg_set_profiling")

    def kernel_stats(self):
        """{class: (total ms, launches, algorithmic bytes)}"""
        k = len(KERNEL_CLASSES)
        ms = np.zeros(k)
        la = np.zeros(k, np.int64)
        by = np.zeros(k)
        self._check(self.lib.ssg_get_kernel_stats(self.h, _p(ms), _p(la), _p(by), k), "ssg_get_kernel_stats")
        return {KERNEL_CLASSES[i]: (float(ms[i]), int(la[i]), float(by[i])) for i in range(k)}

    def set_tuning(self, key, value):
        self._check(self.lib.ssg_set_tuning(self.h, int(key), int(value)), "ssg_set_tuning")

    def autotune(self, keep_group=False):
        """Time the candidate sweep schedules on the current matrix, keep the fastest;
        returns {"mode", "group", "cta_per_sm", "ms"} (ms: one preconditioner application)."""
        m, g, c = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        ms = ctypes.c_double(0.0)
        self._check(self.lib.ssg_autotune(self.h, 1 if keep_group else 0, ctypes.byref(m), ctypes.byref(g),
                                          ctypes.byref(c), ctypes.byref(ms)), "ssg_autotune")
        return {"mode": m.value, "group": g.value, "cta_per_sm": c.value, "ms": ms.value}

    def launch_count(self):
        return int(self.lib.ssg_launch_count())

    def level_schedule(self, lower=True):
        level = np.zeros(max(self.n, 1), np.int32)
        perm = np.zeros(max(self.n, 1), np.int32)
        nlev = ctypes.c_int(0)
        self._check(self.lib.ssg_level_schedule(self.h, 1 if lower else 0, _p(level), _p(perm), ctypes.byref(nlev)),
                    "ssg_level_schedule")
        return level[:self.n], perm[:self.n], nlev.value


class Batch:
    """Many independent systems solved in shared launches (ssg_batch_*)."""

    def __init__(self, device=0):
        from ._native import load_solver
        self.lib = load_solver()
        b = ctypes.c_void_p()
        rc = self.lib.ssg_batch_create(ctypes.byref(b), int(device))
        if rc != SSG_OK:
            raise SolverError(rc, "ssg_batch_create failed")
        self.b = b
        self.systems = []  # (n, nrhs, complex)

    def close(self):
        if getattr(self, "b", None):
            self.lib.ssg_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc < 0:
            msg = self.lib.ssg_batch_last_error(self.b)
            raise SolverError(rc, "%s: %s" % (what, msg.decode() if msg else ""))
        return rc

    def add(self, row_ptr, col, val, B):
        """B: (n,) or (nrhs, n). Returns the system index."""
        rp = np.ascontiguousarray(row_ptr, np.int32)
        ci = np.ascontiguousarray(col, np.int32)
        cplx = np.iscomplexobj(val) or np.iscomplexobj(B)
        dt = np.complex128 if cplx else np.float64
        v = np.ascontiguousarray(val, dt)
        Bm = np.ascontiguousarray(np.atleast_2d(B), dt)
        n = len(rp) - 1
        assert Bm.shape[1] == n
        idx = ctypes.c_int(-1)
        self._check(self.lib.ssg_batch_add(self.b, n, len(ci), _p(rp), _p(ci), _p(v), COMPLEX if cplx else REAL,
                                           Bm.shape[0], _p(Bm), ctypes.byref(idx)), "ssg_batch_add")
        self.systems.append((n, Bm.shape[0], cplx))
        return idx.value

    def set_rhs(self, index, B):
        n, nrhs, cplx = self.systems[index]
        Bm = np.ascontiguousarray(np.atleast_2d(B), np.complex128 if cplx else np.float64)
        assert Bm.shape == (nrhs, n)
        self._check(self.lib.ssg_batch_set_rhs(self.b, int(index), _p(Bm)), "ssg_batch_set_rhs")

    def clear(self):
        self._check(self.lib.ssg_batch_clear(self.b), "ssg_batch_clear")
        self.systems = []

    def start(self, method, alpha, conv=1e-8, max_ite=10000):
        self._check(self.lib.ssg_batch_start(self.b, int(method), float(alpha), float(conv), int(max_ite)),
                    "ssg_batch_start")

    def poll(self):
        d = ctypes.c_int(0)
        self._check(self.lib.ssg_batch_poll(self.b, ctypes.byref(d)), "ssg_batch_poll")
        return bool(d.value)

    def wait(self):
        self._check(self.lib.ssg_batch_wait(self.b), "ssg_batch_wait")

    def step(self):
        """Wait for the iterations in flight, queue more; True once every instance ended."""
        d = ctypes.c_int(0)
        self._check(self.lib.ssg_batch_step(self.b, ctypes.byref(d)), "ssg_batch_step")
        return bool(d.value)

    def finished(self, index):
        f = ctypes.c_int(0)
        self._check(self.lib.ssg_batch_finished(self.b, int(index), ctypes.byref(f)), "ssg_batch_finished")
        return bool(f.value)

    def result(self, index):
        """(X (nrhs, n), iters (nrhs,), status (nrhs,), all converged)"""
        n, nrhs, cplx = self.systems[index]
        X = np.zeros((nrhs, n), np.complex128 if cplx else np.float64)
        it = np.zeros(nrhs, np.int32)
        stt = np.zeros(nrhs, np.int32)
        rc = self._check(self.lib.ssg_batch_result(self.b, int(index), _p(X), _p(it), _p(stt)), "ssg_batch_result")
        return X, it, stt, rc == SSG_OK

    def residual_log(self, index, rhs=0):
        ln = ctypes.c_int(0)
        self._check(self.lib.ssg_batch_residual_log(self.b, int(index), int(rhs), None, 0, ctypes.byref(ln)),
                    "ssg_batch_residual_log")
        out = np.zeros(ln.value)
        self._check(self.lib.ssg_batch_residual_log(self.b, int(index), int(rhs), _p(out), ln.value, ctypes.byref(ln)),
                    "ssg_batch_residual_log")
        return out

    def timings(self):
        t = np.zeros(2)
        self._check(self.lib.ssg_batch_timings(self.b, _p(t)), "ssg_batch_timings")
        return t

    def stream(self):
        s = ctypes.c_void_p()
        self._check(self.lib.ssg_batch_stream(self.b, ctypes.byref(s)), "ssg_batch_stream")
        return s.value or 0

    def set_profiling(self, on):
        self._check(self.lib.ssg_batch_set_profiling(self.b, 1 if on else 0), "ssg_batch_set_profiling")

    def set_graphs(self, on):
        self._check(self.lib.ssg_batch_set_graphs(self.b, 1 if on else 0), "ssg_batch_set_graphs")

    def set_persistent(self, on):
        """FP64 ICCG starts with one CTA per instance running all of its iterations (small systems)."""
        self._check(self.lib.ssg_batch_set_persistent(self.b, 1 if on else 0), "ssg_batch_set_persistent")

    def autotune(self):
        """Times the sweep schedules on the batch and keeps the fastest: {mode, group, cta_per_sm, ms}."""
        m, g, c = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        ms = ctypes.c_double(0.0)
        self._check(self.lib.ssg_batch_autotune(self.b, ctypes.byref(m), ctypes.byref(g), ctypes.byref(c),
                                                ctypes.byref(ms)), "ssg_batch_autotune")
        return {"mode": m.value, "group": g.value, "cta_per_sm": c.value, "ms": ms.value}

    def set_precision(self, precision, inner_tol=0.0):
        self._check(self.lib.ssg_batch_set_precision(self.b, int(precision), float(inner_tol)),
                    "ssg_batch_set_precision")

    def kernel_stats(self):
        """{class: (ms, launches, algorithmic bytes)} since profiling was switched on"""
        k = len(KERNEL_CLASSES)
        ms = np.zeros(k)
        ln = np.zeros(k, np.int64)
        by = np.zeros(k)
        self._check(self.lib.ssg_batch_kernel_stats(self.b, _p(ms), _p(ln), _p(by), k), "ssg_batch_kernel_stats")
        return {c: (float(ms[i]), int(ln[i]), float(by[i])) for i, c in enumerate(KERNEL_CLASSES)}
