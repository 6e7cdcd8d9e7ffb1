"""Device assembly of the voxel systems (ssg_set_matrix_voxel) against the host
generator (voxel/voxelgen.c): pattern, values and right-hand side bit-identical,
real and complex, with the breadth-first and the lexicographic node order and
with Dirichlet faces switched off; maps that do not match the unknown count
are refused before any row is written."""
import ctypes

import numpy as np
import pytest

from sparsesolv_gb300 import _capi, voxel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def handle(gpu):
    h = _capi.Handle(0)
    yield h
    h.close()


def _cases():
    rng = np.random.default_rng(8)
    open_faces = voxel.VoxelCase(7, 6, 5, iron=voxel.seeded_blocks(rng, 5, 1, 2), coils=[voxel.seeded_coil(rng, 5)],
                                 dirichlet_faces=0b100110, order=1)
    return {
        "cc12": voxel.curl_curl_case(12, seed=5, iron_size=4),
        "cfg1": voxel.config1(),
        "ec8": voxel.eddy_current_case(8, seed=4),
        "open_faces_lex": open_faces,
    }


CASES = _cases()


@pytest.mark.parametrize("name", list(CASES))
def test_device_assembly_bit_identical_to_host(handle, name):
    case = CASES[name]
    rp, ci, va, b = case.assemble()
    bd = handle.set_matrix_voxel(case)
    drp, dci, dva = handle.get_matrix()
    assert np.array_equal(drp, rp) and np.array_equal(dci, ci)
    assert dva.dtype == va.dtype and np.array_equal(dva.view(np.float64), va.view(np.float64))
    assert bd.dtype == b.dtype and np.array_equal(bd.view(np.float64), np.asarray(b).view(np.float64))
    assert np.abs(va).max() > 0


def test_device_assembled_system_solves_like_the_host_one(handle):
    case = CASES["cfg1"]
    rp, ci, va, b = case.assemble()
    o = handle.default_options()
    o.accel_factor = 1.1
    handle.set_options(o)
    handle.set_matrix(rp, ci, va)
    x0 = np.zeros_like(b)
    assert handle.solve(_capi.METHOD_ICCG, b, x0, conv=1e-8, max_ite=2000)
    it0 = handle.iters()
    bd = handle.set_matrix_voxel(case)
    x1 = np.zeros_like(bd)
    assert handle.solve(_capi.METHOD_ICCG, bd, x1, conv=1e-8, max_ite=2000)
    assert handle.iters() == it0 and np.array_equal(x1, x0)


def test_device_assembly_refuses_maps_that_do_not_match(handle):
    case = CASES["cc12"]
    ex, ey, ez = case.edge_maps()
    n = int(max(ex.max(), ey.max(), ez.max()) + 1)
    K, M, C = voxel.element_matrices(case.h)
    nu, tz = case.nu(), case.tz()
    P = _capi._p
    for nunk in (n - 1, n + 1):  # an unknown outside the count; an unknown without an edge
        rc = handle.lib.ssg_set_matrix_voxel(handle.h, case.nx, case.ny, case.nz, P(ex), P(ey), P(ez), nunk, P(K),
                                             P(M), P(C), P(nu), None, ctypes.c_double(0.0), P(tz), _capi.REAL, None, 0)
        assert rc == _capi.SSG_ERR_ARG, (nunk, rc)
    # the handle still works
    bd = handle.set_matrix_voxel(case)
    assert np.array_equal(bd, case.assemble()[3])
