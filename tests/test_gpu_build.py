"""CSR from COO triplets on the device (ssg_set_matrix_coo): the same CSR as
the oracle's restatement of the reference's COO constructor, bit for bit
(columns ascending, a repeated entry summed in input order), and a solve on
the matrix built that way equals the solve on the CSR given directly."""
import numpy as np
import pytest

from oracle.oracle import csr_from_coo
from sparsesolv_gb300 import _capi, voxel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def handle(gpu):
    h = _capi.Handle(0)
    yield h
    h.close()


@pytest.mark.parametrize("cplx", [False, True])
def test_device_coo_build_matches_oracle(handle, cplx):
    rng = np.random.default_rng(11 + cplx)
    n, m = 3000, 120_000
    r = rng.integers(0, n, m)
    c = rng.integers(0, n, m)
    r[0], c[0] = n - 1, n - 1
    v = rng.standard_normal(m) * 10.0 ** rng.uniform(-8, 8, m)
    if cplx:
        v = v + 1j * rng.standard_normal(m)
    handle.set_matrix_coo(n, r, c, v)
    rp, ci, va = handle.get_matrix()
    _, _, orp, oci, ova = csr_from_coo(r, c, v)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci) and np.array_equal(va, ova)


def test_solve_on_a_matrix_built_from_shuffled_triplets(handle):
    rp, ci, va, b = voxel.config1().assemble()
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    # every entry twice (its value and an exact zero; either sum is exact), in a random order
    rng = np.random.default_rng(2)
    R = np.concatenate([rows, rows])
    C = np.concatenate([ci, ci])
    V = np.concatenate([va, np.zeros_like(va)])
    order = rng.permutation(len(R))
    handle.set_matrix_coo(n, R[order], C[order], V[order])
    grp, gci, gva = handle.get_matrix()
    assert np.array_equal(grp, rp) and np.array_equal(gci, ci) and np.array_equal(gva, va)
    o = handle.default_options()
    o.accel_factor = 1.1
    handle.set_options(o)
    x1 = np.zeros_like(b)
    assert handle.solve(_capi.METHOD_ICCG, b, x1, conv=1e-8, max_ite=5000)
    it1 = handle.iters()
    handle.set_matrix(rp, ci, va)
    x2 = np.zeros_like(b)
    assert handle.solve(_capi.METHOD_ICCG, b, x2, conv=1e-8, max_ite=5000)
    assert handle.iters() == it1 and np.array_equal(x1, x2)


def test_coo_entries_outside_the_matrix_are_refused(handle):
    with pytest.raises(_capi.SolverError):
        handle.set_matrix_coo(10, np.array([0, 10]), np.array([0, 1]), np.array([1.0, 2.0]))
    with pytest.raises(_capi.SolverError):
        handle.set_matrix_coo(10, np.array([0, -1]), np.array([0, 1]), np.array([1.0, 2.0]))
