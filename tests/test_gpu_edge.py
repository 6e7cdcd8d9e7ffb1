"""Edge cases of the solve path against the FP64 oracle: one unknown, a
diagonal matrix, a chain (one row per level, more levels than the one-cluster
sweep can stage: the sync-free sweep serves it), an arrow matrix with one dense
row (ragged rows, longer than a warp's registers hold, so the factor takes its
in-memory path), a randomly ordered sparse SPD matrix, and two complex-symmetric
systems off the voxel generator (a 2D Laplacian with a complex shift, and the
arrow). Every solve goes through the C ABI, with the automatic sweep choice and
with each schedule forced at the same lanes a row; the forced schedules must give
the same bits.

Parity bar as in the solver tests: real iteration count within 3% (at least 2),
log within 1e-6, x within 1e-6 of the oracle's x, true residual below 1e-7;
complex iteration count within 10%, A x within 5e-8 |b|."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle.oracle import Settings
from sparsesolv_gb300 import _capi

pytestmark = pytest.mark.gpu

METHOD = {"iccg": _capi.METHOD_ICCG, "mrtr": _capi.METHOD_MRTR}


def csr(A):
    A = sp.csr_matrix(A)
    A.sort_indices()
    return (A.indptr.astype(np.int32), A.indices.astype(np.int32),
            np.ascontiguousarray(A.data, np.complex128 if np.iscomplexobj(A.data) else np.float64))


def lap2d(m):
    t = sp.diags([-np.ones(m - 1), 2 * np.ones(m), -np.ones(m - 1)], [-1, 0, 1])
    e = sp.identity(m)
    return sp.kron(t, e) + sp.kron(e, t)


def case(name):
    rng = np.random.default_rng(7)
    if name == "one":
        A = sp.csr_matrix(np.array([[4.0]]))
    elif name == "diagonal":
        A = sp.diags(rng.uniform(0.5, 3.0, 1000))
    elif name == "chain":
        n = 50_000
        A = sp.diags([-np.ones(n - 1), 2.5 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1])
    elif name in ("arrow", "complex_arrow"):
        n = 3000
        A = sp.lil_matrix((n, n))
        A.setdiag(2.0)
        w = rng.uniform(-1.0, 1.0, n - 1) / n
        A[n - 1, : n - 1] = w
        A[: n - 1, n - 1] = w[:, None]
        if name == "complex_arrow":
            A = sp.csr_matrix(A).astype(np.complex128) + 1j * sp.diags(rng.uniform(0.0, 0.2, n))
    elif name == "random_spd":
        n = 20_000
        S = sp.random(n, n, density=5.0 / n, random_state=np.random.RandomState(3), format="csr")
        S = S + S.T
        S.data = -np.abs(S.data)
        d = -np.asarray(S.sum(axis=1)).ravel() + rng.uniform(0.01, 0.1, n)
        A = S + sp.diags(d)
        p = rng.permutation(n)
        A = sp.csr_matrix(A)[p][:, p]
    elif name == "complex":
        K = lap2d(100)
        M = sp.diags(rng.uniform(0.0, 0.05, K.shape[0]))
        A = K.astype(np.complex128) + 1j * M
    else:
        raise KeyError(name)
    rp, ci, va = csr(A)
    n = len(rp) - 1
    b = rng.standard_normal(n)
    if np.iscomplexobj(va):
        b = b + 1j * rng.standard_normal(n)
    return rp, ci, va, b


def solve(h, method, rp, ci, va, b, s, maxit=20000, conv=1e-8):
    h.set_matrix(rp, ci, va)
    o = h.default_options()
    for f, _ in o._fields_:
        if hasattr(s, f):
            setattr(o, f, type(getattr(o, f))(getattr(s, f)))
    h.set_options(o)
    dt = np.complex128 if np.iscomplexobj(va) else np.float64
    x = np.zeros(len(b), dt)
    ok = h.solve(METHOD[method], np.ascontiguousarray(b, dt), x, conv=conv, max_ite=maxit)
    return ok, x, h.residual_log(), h.iters()


REAL = ["one", "diagonal", "chain", "arrow", "random_spd"]
RUNS = [(c, m, pt) for c in REAL for (m, pt) in (("iccg", 1), ("mrtr", 0), ("mrtr", 1))]
RUNS += [("complex", "iccg", 1), ("complex", "mrtr", 0), ("complex_arrow", "iccg", 1)]


@pytest.fixture(scope="module")
def handle(gpu):
    h = _capi.Handle(0)
    yield h
    h.close()


@pytest.mark.parametrize("name,method,pt", RUNS)
def test_edge_case_against_oracle(handle, oracle, name, method, pt):
    rp, ci, va, b = case(name)
    cx = np.iscomplexobj(va)
    s = Settings(accel_factor=1.1, precondition_type=pt, is_save_residual_log=True)
    o = oracle.solve(method, rp, ci, va, b, s, maxit=20000)
    assert o.converged
    ok, x, log, iters = solve(handle, method, rp, ci, va, b, s)   # automatic schedule
    runs = {}
    try:
        # sync-free and one-cluster schedules with the same lanes a row: the same bits
        handle.set_tuning(_capi.TUNE_SWEEP_GROUP, 4)
        handle.set_tuning(_capi.TUNE_CLUSTER_GROUP, 4)
        for mode in (1, 2):
            handle.set_tuning(_capi.TUNE_SWEEP_MODE, mode)
            runs[mode] = solve(handle, method, rp, ci, va, b, s)
    finally:
        handle.set_tuning(_capi.TUNE_SWEEP_MODE, 0)
        handle.set_tuning(_capi.TUNE_SWEEP_GROUP, 0)
        handle.set_tuning(_capi.TUNE_CLUSTER_GROUP, 4)
    assert runs[1][3] == runs[2][3] and np.array_equal(runs[1][1], runs[2][1])
    assert ok and runs[1][0]
    slack = max(2, int((0.10 if cx else 0.03) * o.iters + 0.999))
    assert abs(iters - o.iters) <= slack, (iters, o.iters)
    A = sp.csr_matrix((va, ci, rp))
    if cx:
        assert np.linalg.norm(A @ x - b) <= 5e-8 * np.linalg.norm(b)
    else:
        k = min(len(log), len(o.log), 10)
        assert np.allclose(log[:k], o.log[:k], rtol=1e-6, atol=1e-13 * o.log[0])
        assert np.linalg.norm(x - o.x) <= 1e-6 * np.linalg.norm(o.x)
        assert np.linalg.norm(b - A @ x) < 1e-7 * np.linalg.norm(b)


def test_timeout_reports_error_and_handle_stays_usable(handle, oracle):
    """A bounded wait that runs out: with the spin limit at 1 us the sync-free
    sweep over the 50,000-row chain (each row waits on the one before it, held
    by another warp) gives up, the call returns SSG_ERR_TIMEOUT, and with the
    default limit restored the next solve on the same handle meets the parity
    bar again. No fault and no hang: the wait is cut short, not broken."""
    rp, ci, va, b = case("chain")
    s = Settings(accel_factor=1.1, is_save_residual_log=True)
    o = oracle.solve("iccg", rp, ci, va, b, s, maxit=20000)
    try:
        handle.set_tuning(_capi.TUNE_SWEEP_MODE, 1)
        ok, x, log, iters = solve(handle, "iccg", rp, ci, va, b, s)   # pattern and factor cached
        assert ok and iters == o.iters
        handle.set_tuning(_capi.TUNE_SPIN_LIMIT_US, 1)
        with pytest.raises(_capi.SolverError) as e:
            handle.apply_precond(b)
        assert e.value.code == _capi.SSG_ERR_TIMEOUT
        # a solve that uploads the matrix again re-runs the pattern analysis and the factor,
        # whose waits (level schedule, factor row flags) time out the same way
        with pytest.raises(_capi.SolverError) as e:
            solve(handle, "iccg", rp, ci, va, b, s)
        assert e.value.code == _capi.SSG_ERR_TIMEOUT
    finally:
        handle.set_tuning(_capi.TUNE_SPIN_LIMIT_US, 0)
    try:
        ok, x, log, iters = solve(handle, "iccg", rp, ci, va, b, s)
    finally:
        handle.set_tuning(_capi.TUNE_SWEEP_MODE, 0)
    assert ok and iters == o.iters
    assert np.allclose(log, o.log, rtol=1e-6, atol=1e-13 * o.log[0])
    assert np.linalg.norm(x - o.x) <= 1e-6 * np.linalg.norm(o.x)
