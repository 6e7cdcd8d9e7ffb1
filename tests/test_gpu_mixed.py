"""Mixed precision (SSG_PREC_MIXED): FP32 factor copy, FP32 SpMV and sweeps in
an inner ICCG / IC-MRTR, FP64 refinement on the true residual.

Bar: every result reaches |b - A x| / |b| < 1e-8 (checked here in FP64 on the
host), its error against the FP64 oracle solve is stated and bounded in the
range of A (the curl-curl systems are singular, so x is compared through A x:
|A x - A x_oracle| <= 3e-8 |b|), an instance is bit-identical alone and in a
batch, and the single-system ssg_solve path gives the same as a batch of one."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle.oracle import Settings
from sparsesolv_gb300 import _capi, voxel

pytestmark = pytest.mark.gpu

ALPHA = 1.1
TOL = 1e-8


def true_res(rp, ci, va, b, x):
    A = sp.csr_matrix((va, ci, rp))
    return np.linalg.norm(b - A @ x) / np.linalg.norm(b)


def range_err(rp, ci, va, b, x, xo):
    A = sp.csr_matrix((va, ci, rp))
    return np.linalg.norm(A @ (x - xo)) / np.linalg.norm(b)


def real_systems():
    return [voxel.curl_curl_case(N, seed=s, iron_size=max(2, N // 3)).assemble()
            for N, s in ((8, 1), (12, 2), (10, 3), (16, 4))]


def complex_systems():
    return [voxel.eddy_current_case(N, seed=s).assemble() for N, s in ((6, 3), (8, 4))]


def solve_batch(systems, method, precision=_capi.PREC_MIXED):
    bt = _capi.Batch(0)
    try:
        bt.set_precision(precision)
        for rp, ci, va, b in systems:
            bt.add(rp, ci, va, b)
        bt.start(method, ALPHA, conv=TOL, max_ite=5000)
        bt.wait()
        return [bt.result(k) + (bt.residual_log(k),) for k in range(len(systems))]
    finally:
        bt.close()


@pytest.mark.parametrize("method,name", [(_capi.METHOD_ICCG, "iccg"), (_capi.METHOD_MRTR, "mrtr")])
def test_mixed_real_batch(gpu, oracle, method, name):
    systems = real_systems()
    res = solve_batch(systems, method)
    for (rp, ci, va, b), (X, it, stt, ok, log) in zip(systems, res):
        assert ok and stt[0] == 1
        x = X[0]
        assert true_res(rp, ci, va, b, x) < TOL
        # the refinement log is the true residual after each step, ending below the tolerance
        assert log[0] == 1.0 and log[-1] < TOL and len(log) >= 2
        ores = oracle.solve(name, rp, ci, va, b, Settings(accel_factor=ALPHA, precondition_type=0), conv=TOL)
        assert range_err(rp, ci, va, b, x, ores.x) <= 3e-8
        # the inner iterations stay close to the FP64 count (restarts cost a few)
        assert it[0] <= 1.6 * ores.iters + 10


def test_mixed_complex_mrtr_batch(gpu, oracle):
    systems = complex_systems()
    res = solve_batch(systems, _capi.METHOD_MRTR)
    for (rp, ci, va, b), (X, it, stt, ok, log) in zip(systems, res):
        assert ok
        x = X[0]
        assert true_res(rp, ci, va, b, x) < TOL
        ores = oracle.solve("mrtr", rp, ci, va, b, Settings(accel_factor=ALPHA, precondition_type=0), conv=TOL)
        assert range_err(rp, ci, va, b, x, ores.x) <= 3e-8


def test_mixed_instance_identical_alone_and_in_the_mix(gpu):
    systems = real_systems()
    mix = solve_batch(systems, _capi.METHOD_ICCG)
    for k in (1, 3):
        alone = solve_batch([systems[k]], _capi.METHOD_ICCG)[0]
        assert np.array_equal(alone[0], mix[k][0])
        assert np.array_equal(alone[1], mix[k][1])
        assert np.array_equal(alone[4], mix[k][4])


def test_single_system_solve_with_mixed_precision(gpu):
    rp, ci, va, b = voxel.config1().assemble()
    h = _capi.Handle(0)
    try:
        h.set_matrix(rp, ci, va)
        o = h.default_options()
        o.accel_factor = ALPHA
        o.is_save_residual_log = 1
        o.precision = _capi.PREC_MIXED
        h.set_options(o)
        h.set_tuning(_capi.TUNE_BATCH_GROUP, 8)  # the lanes a row of a user batch, for the bitwise comparison
        for _ in range(2):  # the second call reuses the prepared batch
            x = np.zeros_like(b)
            assert h.solve(_capi.METHOD_ICCG, b, x, conv=TOL, max_ite=5000)
            assert true_res(rp, ci, va, b, x) < TOL
            log = h.residual_log()
            assert log[-1] < TOL and h.iters() > 0
        ref = solve_batch([(rp, ci, va, b)], _capi.METHOD_ICCG)[0]
        # the automatic schedule of a handle's own batch may take the push sweep (its own
        # rounding); a standalone batch keeps to the lane-summed sweeps
        assert range_err(rp, ci, va, b, x, ref[0][0]) <= 3e-8
        # with the lane-summed sweep pinned the handle gives the batch's bits
        h.set_tuning(_capi.TUNE_SWEEP_MODE, 2)
        x = np.zeros_like(b)
        assert h.solve(_capi.METHOD_ICCG, b, x, conv=TOL, max_ite=5000)
        assert np.array_equal(x, ref[0][0])
        h.set_tuning(_capi.TUNE_SWEEP_MODE, 0)
        # unsupported combinations are refused, not approximated
        o.is_diag_scale = 1
        h.set_options(o)
        with pytest.raises(_capi.SolverError):
            h.solve(_capi.METHOD_ICCG, b, np.zeros_like(b), conv=TOL, max_ite=5000)
    finally:
        h.close()
