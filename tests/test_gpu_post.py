"""Flux density B = curl A per voxel (ssg_flux_density): bit-identical to the
oracle's restatement of the reference example's Element::calcB on solved real
and complex systems, and exact on fields whose curl is known."""
import numpy as np
import pytest

from oracle.oracle import flux_density
from sparsesolv_gb300 import _capi, voxel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def handle(gpu):
    h = _capi.Handle(0)
    yield h
    h.close()


@pytest.mark.parametrize("complex_case", [False, True])
def test_flux_density_of_a_solution_matches_oracle(handle, complex_case):
    case = voxel.eddy_current_case(8, seed=4) if complex_case else voxel.curl_curl_case(12, seed=5, iron_size=4)
    rp, ci, va, b = case.assemble()
    handle.set_matrix(rp, ci, va)
    o = handle.default_options()
    o.accel_factor = 1.1
    o.precondition_type = 0
    handle.set_options(o)
    x = np.zeros_like(b)
    assert handle.solve(_capi.METHOD_MRTR if complex_case else _capi.METHOD_ICCG, b, x, conv=1e-8, max_ite=5000)
    B = handle.flux_density(case, x)
    ex, ey, ez = case.edge_maps()
    Bo = flux_density(case.nx, case.ny, case.nz, case.h, ex, ey, ez, x).reshape(B.shape)
    assert np.array_equal(B, Bo)
    assert np.abs(B).max() > 0


def test_flux_density_exact_fields(handle):
    from tests.test_voxel import _interior_fields
    N = 7
    case, ex, ey, ez, grad, unif, B0 = _interior_fields(N, 4)
    Bg = handle.flux_density(case, grad)
    assert np.abs(Bg).max() <= 1e-9 * np.abs(grad).max() / case.h
    Bu = handle.flux_density(case, unif)
    assert np.allclose(Bu[1:-1, 1:-1, 1:-1].reshape(-1, 3), B0[None, :], rtol=1e-12, atol=1e-12)
