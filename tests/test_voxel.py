"""The seeded voxel generator (callers' side): sizes, symmetry, the discrete
de Rham properties that make the curl-curl system singular but consistent,
and the element matrices against closed forms derived independently."""
import numpy as np
import pytest
import scipy.sparse as sp

from sparsesolv_gb300 import voxel


def _gradient(case):
    """Incidence of interior nodes onto unknown edges (edge = end - start)."""
    ex, ey, ez = case.edge_maps()
    nx, ny, nz = case.nx, case.ny, case.nz
    n, _ = case.size()
    lin = lambda x, y, z: x + (nx + 1) * (y + (ny + 1) * z)
    rows, cols, vals = [], [], []
    col = 0
    for z in range(1, nz):
        for y in range(1, ny):
            for x in range(1, nx):
                for emap, d in ((ex, (1, 0, 0)), (ey, (0, 1, 0)), (ez, (0, 0, 1))):
                    out = emap[lin(x, y, z)]              # edge leaving the node (node is its start)
                    inn = emap[lin(x - d[0], y - d[1], z - d[2])]  # edge arriving (node is its end)
                    if out >= 0:
                        rows.append(out); cols.append(col); vals.append(-1.0)
                    if inn >= 0:
                        rows.append(inn); cols.append(col); vals.append(1.0)
                col += 1
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, col))


@pytest.mark.parametrize("N", [3, 5, 8])
def test_sizes_all_faces(N):
    c = voxel.curl_curl_case(N, seed=N)
    n, nnz = c.size()
    assert n == 3 * N * (N - 1) ** 2
    rp, ci, val, b = c.assemble()
    assert len(rp) == n + 1 and rp[-1] == nnz == len(ci)
    assert np.all(np.diff(rp) <= 33) and np.all(np.diff(rp) >= 1)
    for i in range(n):  # sorted, unique, diagonal present
        row = ci[rp[i]:rp[i + 1]]
        assert np.all(np.diff(row) > 0) and i in row


def test_symmetric_and_null_space():
    c = voxel.curl_curl_case(7, seed=3, iron_size=3)
    rp, ci, val, b = c.assemble()
    A = sp.csr_matrix((val, ci, rp))
    assert abs(A - A.T).max() == 0.0
    G = _gradient(c)
    scale = abs(A).max() * 2
    assert abs(A @ G).max() <= 1e-12 * scale      # K G = 0: gradients are in the kernel
    assert np.abs(G.T @ b).max() <= 1e-12 * np.abs(b).max()  # b is divergence free
    assert np.linalg.norm(b) > 0


def test_complex_system():
    c = voxel.eddy_current_case(8, seed=5)
    rp, ci, val, b = c.assemble()
    assert np.iscomplexobj(val)
    A = sp.csr_matrix((val, ci, rp))
    assert abs(A - A.T).max() == 0.0  # complex symmetric (not Hermitian)
    assert np.abs(val.imag).max() > 0
    # mass term only where sigma > 0, and positive semi-definite there
    M = sp.csr_matrix((val.imag, ci, rp))
    x = np.random.default_rng(0).standard_normal(len(b))
    assert x @ (M @ x) >= 0


def test_element_matrices_closed_form():
    h = 2.0e-3
    K, M, C = voxel.element_matrices(h)
    L = h / 2
    # local edge l = 4 d + 2 b + a, transverse signs s1 = 2a-1, s2 = 2b-1
    sig = lambda l: (2 * (l & 1) - 1, 2 * ((l >> 1) & 1) - 1)
    for k in range(4):          # x-edges: transverse (y, z)
        for m in range(4):
            sy_k, sz_k = sig(k)
            sy_m, sz_m = sig(m)
            want = (sz_k * sz_m * L * (2 + 2 * sy_k * sy_m / 3) / (16 * L * L)
                    + sy_k * sy_m * L * (2 + 2 * sz_k * sz_m / 3) / (16 * L * L))
            assert K[k, m] == pytest.approx(want, rel=1e-13)
            # mass: int N_k N_m = 2 (2+2 s s'/3)(2+2 t t'/3) L^3 / (64 L^2)
            wantm = (2 + 2 * sy_k * sy_m / 3) * (2 + 2 * sz_k * sz_m / 3) * L / 32
            assert M[k, m] == pytest.approx(wantm, rel=1e-13)
    assert np.allclose(K, K.T) and np.allclose(M, M.T)
    # x-edges and y-edges are orthogonal in the mass matrix
    assert np.abs(M[0:4, 4:8]).max() == 0.0
    # int N_k . curl N_m for an x-edge k and a y-edge m is -t_m / 8
    for k in range(4):
        for m in range(4, 8):
            tm = 2 * ((m >> 1) & 1) - 1
            assert C[k, m] == pytest.approx(-tm / 8.0, rel=1e-13)


def test_deterministic():
    a = voxel.config1().assemble()
    b = voxel.config1().assemble()
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def test_breadth_first_order_differs_from_lexicographic():
    c = voxel.curl_curl_case(6, seed=1)
    c2 = voxel.curl_curl_case(6, seed=1)
    c2.order = 1
    _, ci1, _, _ = c.assemble()
    _, ci2, _, _ = c2.assemble()
    assert len(ci1) == len(ci2) and not np.array_equal(ci1, ci2)


def test_batched_cases_sizes():
    cases = voxel.batched_cases(count=6, seed=4)
    assert len(cases) == 6
    for case, coils in cases:
        assert 8 <= case.nx <= 32 and len(coils) == 4
        n, _ = case.size()
        B = np.stack([case.rhs(cl) for cl in coils])
        assert B.shape == (4, n) and np.all(np.linalg.norm(B, axis=1) > 0)
