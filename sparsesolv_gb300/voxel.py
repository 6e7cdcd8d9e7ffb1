"""Seeded voxel curl-curl / eddy-current systems (the callers' side of the solver).

The geometry follows the reference's VoxelFEM example: uniform 1 mm voxels,
lowest-order edge elements, reluctivity 1/mu0 in air and 1/(1000 mu0) in iron
(examples/VoxelFEM/Defines_Other.h:220-228, setMaterial.cpp:8-44), and a
T-method source for a rectangular loop current
(examples/VoxelFEM/setT_Vector.cpp:6-60, VoxelMatrix.cpp:24-114). Iron
blocks, conductor blocks and the coil ring are placed from a seed with numpy's
PCG64 generator, which gives the same draws on every platform. All faces carry
n x A = 0 unless ``dirichlet_faces`` says otherwise.

The C assembler (``voxel/voxelgen.c``) does the element integration and the
CSR assembly; this module only decides the geometry.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from ._native import load_voxel

MU0 = 4.0e-7 * math.pi
NU_AIR = 1.0 / MU0
NU_IRON = 1.0 / (1000.0 * MU0)
ALL_FACES = 0x3F


class _Grid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("h", ctypes.c_double), ("dirichlet_faces", ctypes.c_uint), ("order", ctypes.c_int)]


def _lib():
    lib = load_voxel()
    if not getattr(lib, "_declared", False):
        P = ctypes.POINTER
        lib.vx_count.argtypes = [P(_Grid), P(ctypes.c_int64)]
        lib.vx_count.restype = ctypes.c_int64
        lib.vx_assemble.argtypes = [P(_Grid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.vx_assemble.restype = ctypes.c_int64
        lib.vx_edge_maps.argtypes = [P(_Grid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.vx_edge_maps.restype = ctypes.c_int64
        lib.vx_rhs.argtypes = [P(_Grid), ctypes.c_void_p, ctypes.c_void_p]
        lib.vx_rhs.restype = ctypes.c_int64
        lib.vx_element_matrices.argtypes = [ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.vx_element_matrices.restype = None
        lib._declared = True
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class Block:
    """Axis-aligned box of voxels [x0, x0+sx) x [y0, y0+sy) x [z0, z0+sz)."""
    x0: int
    y0: int
    z0: int
    sx: int
    sy: int
    sz: int


@dataclass
class Coil:
    """Rectangular coil ring: outer node box [x0, x1] x [y0, y1], ring width
    ``w`` voxels, carrying current between node planes z0 and z1."""
    x0: int
    y0: int
    x1: int
    y1: int
    w: int
    z0: int
    z1: int
    j0: float = 1.0


@dataclass
class VoxelCase:
    nx: int
    ny: int
    nz: int
    h: float = 1.0e-3
    iron: list = field(default_factory=list)
    conductors: list = field(default_factory=list)
    coils: list = field(default_factory=list)
    sigma: float = 0.0
    omega: float = 0.0
    dirichlet_faces: int = ALL_FACES
    order: int = 0  # 0 = breadth-first node order of the reference mesh maker

    def grid(self):
        return _Grid(self.nx, self.ny, self.nz, self.h, self.dirichlet_faces, self.order)

    # ---- fields on the grid ----
    def nu(self):
        nu = np.full((self.nz, self.ny, self.nx), NU_AIR)
        for b in self.iron:
            nu[b.z0:b.z0 + b.sz, b.y0:b.y0 + b.sy, b.x0:b.x0 + b.sx] = NU_IRON
        return np.ascontiguousarray(nu.reshape(-1))

    def sig(self):
        s = np.zeros((self.nz, self.ny, self.nx))
        for b in self.conductors:
            s[b.z0:b.z0 + b.sz, b.y0:b.y0 + b.sy, b.x0:b.x0 + b.sx] = self.sigma
        return np.ascontiguousarray(s.reshape(-1))

    def tz(self, coils=None):
        """Line integral of T along every z-edge, indexed x + (nx+1)(y + (ny+1) z)."""
        coils = self.coils if coils is None else coils
        t = np.zeros((self.nz, self.ny + 1, self.nx + 1))
        X = np.arange(self.nx + 1)[None, :]
        Y = np.arange(self.ny + 1)[:, None]
        for c in coils:
            d = np.minimum(np.minimum(X - c.x0, c.x1 - X), np.minimum(Y - c.y0, c.y1 - Y))
            d = np.clip(d, 0, c.w).astype(np.float64)
            # T_z = j0 * h * d  [A/m], times the edge length h
            t[c.z0:c.z1, :, :] += c.j0 * self.h * self.h * d[None, :, :]
        return np.ascontiguousarray(t.reshape(-1))

    # ---- assembly ----
    def size(self):
        n = ctypes.c_int64(0)
        g = self.grid()
        nnz = _lib().vx_count(ctypes.byref(g), ctypes.byref(n))
        if nnz < 0:
            raise MemoryError("voxel generator: allocation failed")
        return int(n.value), int(nnz)

    def assemble(self, complex_values=None, coils_list=None):
        """Return (row_ptr, col, val, B): CSR int32/float64 (complex128 when
        the case is complex) and right-hand sides B of shape (n,) or (k, n)."""
        if complex_values is None:
            complex_values = self.sigma != 0.0 and self.omega != 0.0 and bool(self.conductors)
        n, nnz = self.size()
        g = self.grid()
        row_ptr = np.empty(n + 1, np.int32)
        col = np.empty(nnz, np.int32)
        vre = np.empty(nnz, np.float64)
        vim = np.empty(nnz, np.float64) if complex_values else None
        b = np.empty(n, np.float64)
        nu = self.nu()
        sig = self.sig() if complex_values else None
        tz = self.tz()
        got = _lib().vx_assemble(ctypes.byref(g), _ptr(nu), _ptr(sig), float(self.omega), _ptr(tz),
                                 _ptr(row_ptr), _ptr(col), _ptr(vre), _ptr(vim), _ptr(b))
        if got != nnz:
            raise RuntimeError("voxel generator: assembly failed")
        val = vre if vim is None else (vre + 1j * vim)
        if coils_list is None:
            rhs = b if vim is None else b.astype(np.complex128)
        else:
            rhs = np.stack([self.rhs(cl, complex_values) for cl in coils_list])
        return row_ptr, col, val, rhs

    def rhs(self, coils, complex_values=False):
        """Right-hand side for another set of coils on the same matrix."""
        n, _ = self.size()
        g = self.grid()
        b = np.empty(n, np.float64)
        tz = self.tz(coils)
        if _lib().vx_rhs(ctypes.byref(g), _ptr(tz), _ptr(b)) != n:
            raise RuntimeError("voxel generator: rhs assembly failed")
        return b.astype(np.complex128) if complex_values else b

    def edge_maps(self):
        nn = (self.nx + 1) * (self.ny + 1) * (self.nz + 1)
        ex = np.empty(nn, np.int32)
        ey = np.empty(nn, np.int32)
        ez = np.empty(nn, np.int32)
        g = self.grid()
        _lib().vx_edge_maps(ctypes.byref(g), _ptr(ex), _ptr(ey), _ptr(ez))
        return ex, ey, ez


def element_matrices(h=1.0e-3):
    K = np.empty((12, 12))
    M = np.empty((12, 12))
    C = np.empty((12, 12))
    _lib().vx_element_matrices(h, _ptr(K), _ptr(M), _ptr(C))
    return K, M, C


# ---------------------------------------------------------------- seeded cases
def _place(rng, n, size, margin):
    lo = margin
    hi = max(lo, n - margin - size)
    return int(rng.integers(lo, hi + 1))


def seeded_coil(rng, N, nz=None):
    """A coil ring at a seeded position, at least one voxel from every face."""
    nz = N if nz is None else nz
    side = max(4, N // 2)
    w = max(1, N // 10)
    h = max(2, nz // 4)
    x0 = _place(rng, N, side, 1)
    y0 = _place(rng, N, side, 1)
    z0 = _place(rng, nz, h, 1)
    return Coil(x0, y0, x0 + side, y0 + side, w, z0, z0 + h)


def seeded_blocks(rng, N, count, size):
    blocks = []
    for _ in range(count):
        s = min(size, max(1, N - 2))
        blocks.append(Block(_place(rng, N, s, 1), _place(rng, N, s, 1), _place(rng, N, s, 1), s, s, s))
    return blocks


def curl_curl_case(N, seed, n_iron=1, iron_size=6):
    """Static-magnetic curl-curl system on N^3 voxels with ``n_iron`` seeded
    iron blocks of ``iron_size``^3 voxels and one seeded coil ring."""
    rng = np.random.default_rng(seed)
    iron = seeded_blocks(rng, N, n_iron, iron_size)
    coil = seeded_coil(rng, N)
    return VoxelCase(N, N, N, iron=iron, coils=[coil])


def eddy_current_case(N, seed, n_cond=2, cond_size=None, sigma=1.0e7, freq=50.0):
    """Complex-symmetric K + j omega sigma M on N^3 voxels with seeded
    conductor blocks (which are also iron) and one seeded coil ring."""
    rng = np.random.default_rng(seed)
    cs = cond_size if cond_size is not None else max(2, N // 6)
    cond = seeded_blocks(rng, N, n_cond, cs)
    coil = seeded_coil(rng, N)
    return VoxelCase(N, N, N, iron=list(cond), conductors=cond, coils=[coil],
                     sigma=sigma, omega=2.0 * math.pi * freq)


# Workloads the solvers are measured on (sizes and seeds are fixed here).
def config1():
    """20^3 voxels, one 6^3 iron block, coil ring, alpha 1.1, tolerance 1e-8."""
    return curl_curl_case(20, seed=1, n_iron=1, iron_size=6)


def config2():
    """80^3 voxels, three seeded iron blocks."""
    return curl_curl_case(80, seed=2, n_iron=3, iron_size=12)


def config3():
    """60^3 voxels, complex eddy-current system, sigma 1e7 S/m at 50 Hz."""
    return eddy_current_case(60, seed=3)


def batched_cases(count=256, seed=4, lo=8, hi=32, n_rhs=4):
    """``count`` curl-curl systems with N ~ U{lo..hi}, each with ``n_rhs``
    right-hand sides from seeded coil placements."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        N = int(rng.integers(lo, hi + 1))
        sub = int(rng.integers(0, 2**31 - 1))
        case = curl_curl_case(N, seed=sub, n_iron=1, iron_size=max(2, N // 4))
        r2 = np.random.default_rng(sub + 1)
        coils = [[seeded_coil(r2, N)] for _ in range(n_rhs)]
        out.append((case, coils))
    return out
