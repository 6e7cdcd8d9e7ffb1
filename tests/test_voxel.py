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


def _interior_fields(N, seed):
    """A gradient field and the field of a uniform B0 on the edges of an N^3 case."""
    case = voxel.curl_curl_case(N, seed=seed, iron_size=2)
    ex, ey, ez = case.edge_maps()
    n = int(max(ex.max(), ey.max(), ez.max())) + 1
    h = case.h
    P = np.arange(N + 1) * h
    Z, Y, X = np.meshgrid(P, P, P, indexing="ij")
    X, Y, Z = X.ravel(), Y.ravel(), Z.ravel()
    rng = np.random.default_rng(seed)
    # zero on the boundary, whose edges carry no unknown (n x A = 0 there)
    on_bnd = (X == 0) | (Y == 0) | (Z == 0) | (X == P[-1]) | (Y == P[-1]) | (Z == P[-1])
    phi = np.where(on_bnd, 0.0, rng.standard_normal(X.size))
    B0 = np.array([0.3, -0.7, 1.1])
    grad = np.zeros(n)
    unif = np.zeros(n)
    stride = {0: 1, 1: N + 1, 2: (N + 1) ** 2}
    for d, m in enumerate((ex, ey, ez)):
        nodes = np.flatnonzero(m >= 0)
        grad[m[nodes]] = phi[nodes + stride[d]] - phi[nodes]
        # A = B0 x r / 2 is linear, so its edge integral is A(midpoint) . e_d h
        mid = np.stack([X[nodes], Y[nodes], Z[nodes]], 1)
        mid[:, d] += h / 2
        unif[m[nodes]] = 0.5 * np.cross(B0, mid)[:, d] * h
    return case, ex, ey, ez, grad, unif, B0


def test_flux_density_restatement_on_exact_fields():
    """curl of a gradient is zero; a uniform field is reproduced in every element
    whose 12 edges all carry unknowns (the boundary edges are Dirichlet)."""
    from oracle.oracle import flux_density
    N = 6
    case, ex, ey, ez, grad, unif, B0 = _interior_fields(N, 3)
    Bg = flux_density(N, N, N, case.h, ex, ey, ez, grad)
    assert np.abs(Bg).max() <= 1e-9 * np.abs(grad).max() / case.h
    Bu = flux_density(N, N, N, case.h, ex, ey, ez, unif).reshape(N, N, N, 3)
    inner = Bu[1:-1, 1:-1, 1:-1].reshape(-1, 3)
    assert np.allclose(inner, B0[None, :], rtol=1e-12, atol=1e-12)
