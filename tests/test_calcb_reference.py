"""Pins the oracle's B = curl A (oracle.flux_density, the checker of the GPU's
ssg_flux_density) against the reference example's own code, on the CPU:
the example's mesh maker (examples/VoxelFEM/MeshMakerFile/MeshMaker.h) builds
the voxel mesh, and its Element::calcB (examples/VoxelFEM/Element.cpp:47-90)
computes the element-centre flux density from a seeded A, both compiled out of
tree by `make -C oracle calcb` (shims in oracle/calcb/). Each of the
reference's edges gets the matrix index this repository's generator gives the
same physical edge (boundary edges after the unknowns, with A = 0, as the
example's VoxelMesh::setSubIDs orders them). Skipped without a reference
checkout."""
import os
import subprocess

import numpy as np
import pytest

from oracle.oracle import flux_density
from sparsesolv_gb300 import voxel

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(REPO, "oracle", "_ref")


@pytest.fixture(scope="module")
def shims():
    r = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "calcb"], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("reference example not available: " + (r.stderr.strip().splitlines() or ["make failed"])[-1])
    return os.path.join(REF, "mesh_shim"), os.path.join(REF, "calcb_shim")


@pytest.mark.parametrize("N,seed", [(7, 3), (5, 11)])
def test_oracle_flux_density_matches_reference_calcb(tmp_path, shims, N, seed):
    mesh_shim, calcb_shim = shims
    case = voxel.curl_curl_case(N, seed=seed, iron_size=2)
    nx, ny, nz, h = case.nx, case.ny, case.nz, case.h
    ex, ey, ez = case.edge_maps()
    n = case.size()[0]
    run = tmp_path / "run"
    run.mkdir()
    (tmp_path / "MeshData").mkdir()
    subprocess.run([mesh_shim, str(nx), str(ny), str(nz), repr(h)], cwd=run, check=True, capture_output=True)
    md = tmp_path / "MeshData"
    with open(md / "Node.vxldata") as f:
        head = f.readline().split()
        assert [int(v) for v in head[1:]] == [nx, ny, nz]
        nodes = np.loadtxt(f, ndmin=2)
    order = np.argsort(nodes[:, 0])
    grid = np.rint(nodes[order, 1:4] / h).astype(np.int64)  # node id -> (i, j, k)
    assert np.allclose(nodes[order, 1:4], grid * h, rtol=0, atol=1e-12)
    with open(md / "Edge.vxldata") as f:
        ne = int(f.readline())
        edges = np.loadtxt(f, dtype=np.int64, ndmin=2)
    assert len(edges) == ne
    edges = edges[np.argsort(edges[:, 0])]
    s, e = grid[edges[:, 1]], grid[edges[:, 2]]
    lo = np.minimum(s, e)
    d = np.abs(e - s)
    assert np.all(d.sum(axis=1) == 1)  # unit edges along one axis
    lin = lo[:, 0] + (nx + 1) * (lo[:, 1] + (ny + 1) * lo[:, 2])
    ours = np.where(d[:, 0] == 1, ex[lin], np.where(d[:, 1] == 1, ey[lin], ez[lin]))
    known = ours >= 0
    assert np.array_equal(np.sort(ours[known]), np.arange(n))  # every unknown is exactly one reference edge
    sub = ours.copy()
    sub[~known] = n + np.arange((~known).sum())
    np.savetxt(tmp_path / "subid.txt", sub, fmt="%d")
    A = np.random.default_rng(seed).standard_normal(n)
    np.concatenate([A, np.zeros((~known).sum())]).tofile(tmp_path / "A.bin")
    subprocess.run([calcb_shim, str(md), str(tmp_path / "subid.txt"), str(tmp_path / "A.bin"),
                    str(tmp_path / "B.bin")], check=True)
    rec = np.fromfile(tmp_path / "B.bin", dtype=np.dtype([("xyz", "<i4", 3), ("B", "<f8", 6)]))
    assert len(rec) == nx * ny * nz
    x, y, z = rec["xyz"].T
    Bo = flux_density(nx, ny, nz, h, ex, ey, ez, A)[x + nx * (y + ny * z)]
    Br = rec["B"]
    assert np.allclose(Br[:, :3], (np.stack([x, y, z], 1) + 0.5) * h, rtol=1e-12, atol=0)
    # the reference takes the half cell sizes from node coordinates ((x+1)h - xh) / 2, the
    # restatement h / 2; on these meshes the two agree bit for bit
    assert np.abs(Br[:, 3:]).max() > 0
    assert np.array_equal(Br[:, 3:], Bo), np.abs(Br[:, 3:] - Bo).max()
