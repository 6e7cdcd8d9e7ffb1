"""GPU parity of the hot-path pieces, through the C ABI, against the oracle:
level sets and level permutation (bit-exact), IC(0) factor, the IC
preconditioner sweeps, SpMV."""
import numpy as np
import pytest
import scipy.sparse as sp

from sparsesolv_gb300 import _capi
from sparsesolv_gb300 import voxel

pytestmark = pytest.mark.gpu


def _random_spd_pattern(n, density, seed, cplx=False):
    rng = np.random.default_rng(seed)
    A = sp.random(n, n, density=density, random_state=rng, format="csr")
    A = A + A.T + sp.eye(n) * (n * 0.5)
    A = A.tocsr()
    A.sort_indices()
    val = A.data.astype(np.complex128) * (1 + 0.1j) if cplx else A.data
    return A.indptr.astype(np.int32), A.indices.astype(np.int32), val


def _cases():
    out = {}
    out["cc8"] = voxel.curl_curl_case(8, seed=21).assemble()[:3]
    out["cfg1"] = voxel.config1().assemble()[:3]
    out["rand"] = _random_spd_pattern(3000, 0.002, 5)
    out["ec6"] = voxel.eddy_current_case(6, seed=9).assemble()[:3]
    out["rand_c"] = _random_spd_pattern(1500, 0.004, 6, cplx=True)
    return out


CASES = _cases()


@pytest.fixture(scope="module")
def handle(gpu):
    h = _capi.Handle(0)
    yield h
    h.close()


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("lower", [True, False])
def test_level_schedule_bit_exact(handle, oracle, name, lower):
    rp, ci, val = CASES[name]
    handle.set_matrix(rp, ci, val)
    level, perm, nlev = handle.level_schedule(lower)
    trp, tci, _ = oracle.triangle(rp, ci, lower)
    olevel, operm, olptr = oracle.levels(trp, tci, lower)
    assert nlev == len(olptr) - 1
    assert np.array_equal(level, olevel)
    assert np.array_equal(perm, operm)


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("alpha", [1.0, 1.1, 1.3])
def test_ic_factor(handle, oracle, name, alpha):
    rp, ci, val = CASES[name]
    handle.set_matrix(rp, ci, val)
    lrp, lci, lval, D = handle.factor(alpha)
    orp, oci, oval, oD = oracle.ic_factor(rp, ci, val, alpha)
    assert np.array_equal(lrp, orp) and np.array_equal(lci, oci)   # integer pattern: bit-exact
    scale = np.abs(oval).max()
    # alpha = 1 on the singular curl-curl matrices drives pivots towards zero and
    # amplifies last-bit differences of the (reordered) sums; the reference and
    # the oracle differ the same way there
    rtol = 1e-5 if alpha == 1.0 else 1e-9
    assert np.allclose(lval, oval, rtol=rtol, atol=1e-12 * scale)
    assert np.allclose(D, oD, rtol=rtol, atol=0)


@pytest.mark.parametrize("name", list(CASES))
def test_ic_preconditioner_apply(handle, oracle, name):
    rp, ci, val = CASES[name]
    handle.set_matrix(rp, ci, val)
    lrp, lci, lval, D = handle.factor(1.1)
    rng = np.random.default_rng(1)
    n = len(rp) - 1
    r = rng.standard_normal(n)
    if np.iscomplexobj(val):
        r = r + 1j * rng.standard_normal(n)
    z = handle.apply_precond(r)
    zo = oracle.ic_apply(lrp, lci, lval, D, r)   # oracle substitution on the GPU's factor
    assert np.linalg.norm(z - zo) <= 1e-11 * np.linalg.norm(zo)


@pytest.mark.parametrize("mode", [1, 2, 3, 4])
@pytest.mark.parametrize("name", list(CASES))
def test_ic_apply_every_schedule(handle, oracle, name, mode):
    """Every sweep schedule (sync-free, lockstep cluster, neighbour-synchronised,
    push) against the oracle's substitution on the same factor, and the same
    bits on a second apply (deterministic). The push sweep sums each row in
    dependency-level order, so it agrees with the others at rounding level."""
    rp, ci, val = CASES[name]
    handle.set_matrix(rp, ci, val)
    lrp, lci, lval, D = handle.factor(1.1)
    rng = np.random.default_rng(6)
    n = len(rp) - 1
    r = rng.standard_normal(n)
    if np.iscomplexobj(val):
        r = r + 1j * rng.standard_normal(n)
    try:
        handle.set_tuning(_capi.TUNE_SWEEP_MODE, mode)
        z = handle.apply_precond(r)
        z2 = handle.apply_precond(r)
    finally:
        handle.set_tuning(_capi.TUNE_SWEEP_MODE, 0)
    zo = oracle.ic_apply(lrp, lci, lval, D, r)
    assert np.linalg.norm(z - zo) <= 1e-11 * np.linalg.norm(zo)
    assert np.array_equal(z, z2)


@pytest.mark.parametrize("name", list(CASES))
def test_spmv(handle, oracle, name):
    rp, ci, val = CASES[name]
    handle.set_matrix(rp, ci, val)
    n = len(rp) - 1
    x = np.random.default_rng(2).standard_normal(n)
    if np.iscomplexobj(val):
        x = x * (1 - 0.5j)
    y = handle.spmv(x)
    yo = oracle.spmv(rp, ci, val, x)
    assert np.allclose(y, yo, rtol=1e-13, atol=1e-13 * np.abs(yo).max())


def test_missing_diagonal_reports_error(handle):
    rp = np.array([0, 1, 2, 4], np.int32)
    ci = np.array([0, 1, 0, 1], np.int32)  # row 2 lacks its diagonal
    handle.set_matrix(rp, ci, np.array([2.0, 2.0, 1.0, 1.0]))
    with pytest.raises(_capi.SolverError) as e:
        handle.factor(1.0)
    assert e.value.code == _capi.SSG_ERR_NO_DIAGONAL
    # the handle stays usable
    rp, ci, val = CASES["cc8"]
    handle.set_matrix(rp, ci, val)
    handle.factor(1.1)


def test_factor_golden_fixture(handle, golden, golden_cases):
    data, meta = golden
    for key in ["doc5/ic1.00", "doc5/ic1.10", "cc6/ic1.10", "ec5/ic1.10"]:
        rp, ci, va, b = golden_cases[key.split("/")[0]]
        handle.set_matrix(rp, ci, va)
        lrp, lci, lval, D = handle.factor(meta["factors"][key]["alpha"])
        assert np.array_equal(lrp, data[key + "/lrp"]) and np.array_equal(lci, data[key + "/lci"])
        assert np.allclose(lval, data[key + "/lval"], rtol=1e-9, atol=1e-12 * np.abs(lval).max())
        assert np.allclose(D, data[key + "/D"], rtol=1e-9)


@pytest.mark.parametrize("name", ["cc8", "cfg1", "rand"])
@pytest.mark.parametrize("alpha", [1.0, 1.1])
def test_ic_factor_real_bit_identical(handle, oracle, name, alpha):
    """The real factor repeats the reference's operations in the reference's
    order without FMA contraction, so it matches the oracle (itself
    bit-identical to the reference's IC_decomp) exactly."""
    rp, ci, val = CASES[name]
    handle.set_matrix(rp, ci, val)
    _, _, lval, D = handle.factor(alpha)
    _, _, oval, oD = oracle.ic_factor(rp, ci, val, alpha)
    assert np.array_equal(lval, oval) and np.array_equal(D, oD)


@pytest.mark.parametrize("name", ["cc8", "cfg1", "rand", "ec6"])
def test_cluster_and_syncfree_sweeps_agree(handle, name):
    """The one-cluster sweeps (level-synchronous and neighbour-synchronised) and
    the sync-free sweep do the same per-row arithmetic (same lanes, same order),
    so the preconditioner results are identical."""
    rp, ci, val = CASES[name]
    handle.set_matrix(rp, ci, val)
    handle.factor(1.1)
    n = len(rp) - 1
    r = np.random.default_rng(3).standard_normal(n)
    if np.iscomplexobj(val):
        r = r + 0.5j * np.random.default_rng(4).standard_normal(n)
    out = {}
    for g in (4, 8):
        handle.set_tuning(_capi.TUNE_SWEEP_GROUP, g)
        handle.set_tuning(_capi.TUNE_CLUSTER_GROUP, g)
        for mode in (1, 2, 3):
            handle.set_tuning(_capi.TUNE_SWEEP_MODE, mode)
            out[mode, g] = handle.apply_precond(r)
        assert np.array_equal(out[1, g], out[2, g])
        assert np.array_equal(out[1, g], out[3, g])
    handle.set_tuning(_capi.TUNE_SWEEP_MODE, 0)
    handle.set_tuning(_capi.TUNE_SWEEP_GROUP, 0)
    handle.set_tuning(_capi.TUNE_CLUSTER_GROUP, 4)


def test_switching_sweep_modes_replans(handle):
    """Mode 3 then mode 2 on one handle: the second must run the lockstep plan
    (the same results either way; the timing of the lockstep plan is checked
    against a fresh handle elsewhere), and the switch must not fail."""
    rp, ci, val = CASES["cc8"]
    handle.set_matrix(rp, ci, val)
    handle.factor(1.1)
    r = np.random.default_rng(5).standard_normal(len(rp) - 1)
    try:
        handle.set_tuning(_capi.TUNE_SWEEP_MODE, 3)
        z3 = handle.apply_precond(r)
        handle.set_tuning(_capi.TUNE_SWEEP_MODE, 2)
        z2 = handle.apply_precond(r)
        handle.set_tuning(_capi.TUNE_SWEEP_MODE, 3)
        z3b = handle.apply_precond(r)
        assert np.array_equal(z3, z2) and np.array_equal(z3, z3b)
    finally:
        handle.set_tuning(_capi.TUNE_SWEEP_MODE, 0)
