"""ssg_solve_multi: several right-hand sides of one matrix in one call.

With the settings a batch takes, the right-hand sides run as instances of a
one-system batch (one factor, shared launches). Each must then meet the solver
parity bar against a separate ssg_solve of the same right-hand side: iteration
count within 3% (real) / 10% (complex), x within 1e-6 relative (real), true
residual below 1e-7 (real) / A x within 5e-8 |b| (complex). In mixed precision a
single solve is itself a one-system batch, so with the lanes a row pinned the
results must be the same bits.
With other settings the right-hand sides are solved one after another by the
single-system path: the same bits as separate ssg_solve calls."""
import numpy as np
import pytest
import scipy.sparse as sp

from sparsesolv_gb300 import _capi

pytestmark = pytest.mark.gpu

METHOD = {"iccg": _capi.METHOD_ICCG, "mrtr": _capi.METHOD_MRTR}


@pytest.fixture(scope="module")
def handle(gpu):
    h = _capi.Handle(0)
    yield h
    h.close()


def rhs_set(rp, ci, va, b, k, seed=11):
    """b and k - 1 right-hand sides in the range of A (the curl-curl systems are
    singular: a consistent right-hand side needs one), scaled to |b|."""
    A = sp.csr_matrix((va, ci, rp))
    rng = np.random.default_rng(seed)
    out = [b]
    for _ in range(k - 1):
        v = rng.standard_normal(len(b))
        if np.iscomplexobj(va):
            v = v + 1j * rng.standard_normal(len(b))
        e = A @ v
        out.append(e * (np.linalg.norm(b) / np.linalg.norm(e)))
    return np.ascontiguousarray(np.stack(out))


def set_opts(h, **kw):
    o = h.default_options()
    o.accel_factor = 1.1
    o.precondition_type = 0
    o.is_save_residual_log = 1
    for k, v in kw.items():
        setattr(o, k, v)
    h.set_options(o)


def single(h, method, b, x0=None):
    x = np.zeros_like(b) if x0 is None else x0.copy()
    ok = h.solve(METHOD[method], np.ascontiguousarray(b), x, conv=1e-8, max_ite=5000)
    return ok, x, h.iters()


@pytest.mark.parametrize("key,method", [("cfg1", "iccg"), ("cfg1", "mrtr"), ("ec8", "iccg"), ("ec8", "mrtr")])
def test_multi_rhs_meets_the_single_solve_bar(handle, golden_cases, key, method):
    rp, ci, va, b = golden_cases[key]
    cx = np.iscomplexobj(va)
    handle.set_matrix(rp, ci, va)
    set_opts(handle)
    B = rhs_set(rp, ci, va, b, 4)
    X = np.zeros_like(B)
    ok, it, st = handle.solve_multi(METHOD[method], B, X, conv=1e-8, max_ite=5000)
    assert ok and np.all(st == _capi.SSG_OK)
    assert len(handle.residual_log()) == it[-1] + 1   # the log of the last right-hand side
    A = sp.csr_matrix((va, ci, rp))
    for j in range(len(B)):
        ok1, xs, its = single(handle, method, B[j])
        assert ok1
        assert abs(int(it[j]) - its) <= max(2, int((0.10 if cx else 0.03) * its + 0.999)), (j, it[j], its)
        if cx:
            assert np.linalg.norm(A @ X[j] - B[j]) <= 5e-8 * np.linalg.norm(B[j])
        else:
            assert np.linalg.norm(X[j] - xs) <= 1e-6 * np.linalg.norm(xs)
            assert np.linalg.norm(B[j] - A @ X[j]) < 1e-7 * np.linalg.norm(B[j])


def test_multi_rhs_mixed_precision_same_bits_as_single(handle, golden_cases):
    rp, ci, va, b = golden_cases["cfg1"]
    handle.set_matrix(rp, ci, va)
    set_opts(handle, precision=_capi.PREC_MIXED)
    handle.set_tuning(_capi.TUNE_BATCH_GROUP, 8)  # one lane count for one and several right-hand sides
    try:
        B = rhs_set(rp, ci, va, b, 3)
        X = np.zeros_like(B)
        ok, it, st = handle.solve_multi(_capi.METHOD_ICCG, B, X)
        assert ok
        for j in range(len(B)):
            ok1, xs, its = single(handle, "iccg", B[j])
            assert ok1 and its == it[j] and np.array_equal(xs, X[j])
    finally:
        handle.set_tuning(_capi.TUNE_BATCH_GROUP, 0)
        set_opts(handle)


@pytest.mark.parametrize("over", [dict(is_diag_scale=1), dict(is_save_best=1), dict(is_init=0)])
def test_other_settings_solve_one_after_another(handle, golden_cases, over):
    rp, ci, va, b = golden_cases["cc10"]
    handle.set_matrix(rp, ci, va)
    B = rhs_set(rp, ci, va, b, 3)
    X0 = np.zeros_like(B)
    if over.get("is_init") == 0:
        # a warm start: half of each solution (the system is singular: a guess off the
        # range of the solutions can leave a residual the tolerance cannot reach)
        set_opts(handle)
        for j in range(len(B)):
            X0[j] = 0.5 * single(handle, "iccg", B[j])[1]
    set_opts(handle, **over)
    try:
        X = X0.copy()
        ok, it, st = handle.solve_multi(_capi.METHOD_ICCG, B, X)
        assert ok
        for j in range(len(B)):
            ok1, xs, its = single(handle, "iccg", B[j], X0[j])
            assert ok1 and its == it[j] and np.array_equal(xs, X[j])
    finally:
        set_opts(handle)


def test_multi_rhs_argument_checks(handle, golden_cases):
    rp, ci, va, b = golden_cases["cc10"]
    handle.set_matrix(rp, ci, va)
    set_opts(handle)
    lib = handle.lib
    assert lib.ssg_solve_multi(handle.h, _capi.METHOD_ICCG, 1e-8, 100, -1, None, None, None, None) == _capi.SSG_ERR_ARG
    assert lib.ssg_solve_multi(handle.h, _capi.METHOD_ICCG, 1e-8, 100, 0, None, None, None, None) == _capi.SSG_OK
    assert lib.ssg_solve_multi(handle.h, 7, 1e-8, 100, 1, None, None, None, None) == _capi.SSG_ERR_ARG
