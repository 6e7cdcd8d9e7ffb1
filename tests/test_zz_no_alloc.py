"""ssg_ic_factor_noalloc: the IC(0) factor for callers that may not allocate
device memory (code under an external memory manager that owns every device
byte, or a real-time loop where an allocation's latency or failure is not
allowed). Its scratch is a file-scope array of the library, shared by every
call, so the checks run two calls in a row on the same scratch.

Checked against the oracle's restatement of the reference's IC_decomp (real:
bit for bit, as the handle's factor is), against the reference's own complex
factor (golden fixture), against the existing entry point (ssg_factor on a
handle), and on the error returns the kernel reports as status. Named to be
collected last."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from sparsesolv_gb300 import _capi, voxel


def lower_part(rp, ci, val):
    """Lower triangle (diagonal included) of a CSR matrix with sorted rows."""
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    keep = ci <= rows
    lrp = np.zeros(n + 1, np.int32)
    np.cumsum(np.bincount(rows[keep], minlength=n), out=lrp[1:])
    return lrp, np.ascontiguousarray(ci[keep], np.int32), np.ascontiguousarray(val[keep])


def test_noalloc_rejects_bad_sizes_before_touching_the_gpu(solver_lib):
    f = solver_lib.ssg_ic_factor_noalloc
    big = _capi.NOALLOC_MAX_ROWS + 1
    assert f(big, 17 * big, None, None, None, None, None, 1.1, _capi.REAL, None) == _capi.SSG_ERR_ARG
    assert f(10, 30, None, None, None, None, None, 0.0, _capi.REAL, None) == _capi.SSG_ERR_ARG
    assert f(10, 30, None, None, None, None, None, 1.1, 7, None) == _capi.SSG_ERR_ARG
    assert f(0, 0, None, None, None, None, None, 1.1, _capi.REAL, None) == _capi.SSG_OK
    # misaligned pointers are refused by value, before anything reads them: a complex
    # value is one 16-byte load, a real one 8 bytes, the pattern 4 bytes
    P = ctypes.c_void_p
    a16, a8, a2 = P(0x10000), P(0x10008), P(0x10002)
    assert f(10, 30, a16, a16, a8, a16, a16, 1.1, _capi.COMPLEX, None) == _capi.SSG_ERR_ARG
    assert f(10, 30, a16, a16, a16, a8, a16, 1.1, _capi.COMPLEX, None) == _capi.SSG_ERR_ARG
    assert f(10, 30, a16, a16, a16, a16, a8, 1.1, _capi.COMPLEX, None) == _capi.SSG_ERR_ARG
    assert f(10, 30, a2, a16, a8, a8, a8, 1.1, _capi.REAL, None) == _capi.SSG_ERR_ARG
    assert f(10, 30, a16, a16, a2, a8, a8, 1.1, _capi.REAL, None) == _capi.SSG_ERR_ARG


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class _Dev:
    """Device copies of a lower-triangle pattern and values, outputs, stream."""

    def __init__(self, lrp, lci, lval):
        import torch
        self.dev = torch.device("cuda", 0)
        torch.cuda.set_device(self.dev)
        self.n = len(lrp) - 1
        self.nnz = len(lci)
        self.lrp = torch.from_numpy(np.ascontiguousarray(lrp, np.int32)).to(self.dev)
        self.lci = torch.from_numpy(np.ascontiguousarray(lci, np.int32)).to(self.dev)
        self.val = torch.from_numpy(np.ascontiguousarray(lval)).to(self.dev)
        self.out = torch.empty_like(self.val)
        self.D = torch.empty(max(self.n, 1), dtype=self.val.dtype, device=self.dev)
        self.vtype = _capi.COMPLEX if np.iscomplexobj(lval) else _capi.REAL
        self.stream = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def call(self, lib, alpha, inplace=False):
        self.out.fill_(float("nan"))
        self.D.fill_(float("nan"))
        if inplace:
            self.out.copy_(self.val)
        src = self.out if inplace else self.val
        rc = lib.ssg_ic_factor_noalloc(self.n, self.nnz, _ptr(self.lrp), _ptr(self.lci), _ptr(src), _ptr(self.out),
                                       _ptr(self.D), alpha, self.vtype, self.stream)
        return rc, self.out.cpu().numpy(), self.D.cpu().numpy()[:self.n]


@pytest.mark.gpu
def test_noalloc_real_factor_bit_identical_to_oracle_and_handle(oracle):
    rp, ci, val, _ = voxel.config1().assemble()
    lrp, lci, lval = lower_part(rp, ci, val)
    d = _Dev(lrp, lci, lval)
    h = _capi.Handle(0)
    try:
        h.set_matrix(rp, ci, val)
        for alpha in (1.1, 1.05):  # two calls in a row, the second on the first one's scratch
            rc, L, D = d.call(h.lib, alpha)
            assert rc == _capi.SSG_OK, rc
            olrp, olci, oval, oD = oracle.ic_factor(rp, ci, val, alpha)
            assert np.array_equal(olrp, lrp) and np.array_equal(olci, lci)
            assert np.array_equal(L, oval) and np.array_equal(D, oD)
            # the existing entry point (a handle's factor) gives the same bits
            _, _, hval, hD = h.factor(alpha)
            assert np.array_equal(L, hval) and np.array_equal(D, hD)
        rc, L, D = d.call(h.lib, 1.05, inplace=True)  # lval may be the input array
        assert rc == _capi.SSG_OK and np.array_equal(L, oval) and np.array_equal(D, oD)
    finally:
        h.close()


@pytest.mark.gpu
def test_noalloc_complex_factor_matches_reference_and_handle(golden, golden_cases):
    """Complex: the reference divides with libgcc's complex division, the
    kernels with Smith's algorithm, so the factor agrees with the reference to
    rounding (1e-12) rather than bit for bit; with the handle's factor it is
    exact."""
    data, meta = golden
    rp, ci, val, _ = golden_cases["ec5"]
    lrp, lci, lval = lower_part(rp, ci, val)
    d = _Dev(lrp, lci, lval)
    h = _capi.Handle(0)
    try:
        h.set_matrix(rp, ci, val)
        for _ in range(2):
            rc, L, D = d.call(h.lib, 1.1)
            assert rc == _capi.SSG_OK, rc
            assert np.array_equal(lrp, data["ec5/ic1.10/lrp"]) and np.array_equal(lci, data["ec5/ic1.10/lci"])
            gL, gD = data["ec5/ic1.10/lval"], data["ec5/ic1.10/D"]
            assert np.abs(L - gL).max() <= 1e-12 * np.abs(gL).max()
            assert np.all(np.abs(D - gD) <= 1e-12 * np.abs(gD))
            _, _, hval, hD = h.factor(1.1)
            assert np.array_equal(L, hval) and np.array_equal(D, hD)
    finally:
        h.close()


def _spd_lower(n, extra_row=None):
    """Lower triangle of a small diagonally dominant tridiagonal matrix; row
    `extra_row` (if given) couples to every earlier row."""
    rows = []
    for i in range(n):
        if extra_row is not None and i == extra_row:
            cols = list(range(i + 1))
        else:
            cols = [i - 1, i] if i > 0 else [0]
        rows.append(cols)
    lrp = np.zeros(n + 1, np.int32)
    lrp[1:] = np.cumsum([len(r) for r in rows])
    lci = np.array([c for r in rows for c in r], np.int32)
    lval = np.array([4.0 + len(r) if c == i else -1.0 for i, r in enumerate(rows) for c in r])
    return lrp, lci, lval


@pytest.mark.gpu
def test_noalloc_error_returns_then_a_good_call():
    """Host-built bad patterns the kernel reports as status (nothing out of
    bounds is read), each followed by a good call on the same scratch."""
    lrp, lci, lval = _spd_lower(10)
    h = _capi.Handle(0)
    try:
        n = 10
        rows = np.repeat(np.arange(n), np.diff(lrp))
        full = {}
        for r, c, v in zip(rows, lci, lval):
            full[(r, c)] = v
            full[(c, r)] = v
        keys = sorted(full)
        rp = np.zeros(n + 1, np.int32)
        np.cumsum(np.bincount([k[0] for k in keys], minlength=n), out=rp[1:])
        ci = np.array([k[1] for k in keys], np.int32)
        va = np.array([full[k] for k in keys])
        h.set_matrix(rp, ci, va)
        _, _, hval, hD = h.factor(1.1)

        def good():
            rc, L, D = _Dev(lrp, lci, lval).call(h.lib, 1.1)
            assert rc == _capi.SSG_OK and np.array_equal(L, hval) and np.array_equal(D, hD)

        good()
        # row 5 without its diagonal: its columns are 2, 3
        bad_ci = lci.copy()
        bad_ci[lrp[6] - 1] = 3
        bad_ci[lrp[6] - 2] = 2
        assert _Dev(lrp, bad_ci, lval).call(h.lib, 1.1)[0] == _capi.SSG_ERR_NO_DIAGONAL
        good()
        # an off-diagonal column beyond the row (row 7 reads column 8)
        bad_ci = lci.copy()
        bad_ci[lrp[7]] = 8
        bad_ci[lrp[7] + 1] = 7
        assert _Dev(lrp, bad_ci, lval).call(h.lib, 1.1)[0] == _capi.SSG_ERR_ARG
        good()
        # columns not ascending: row 9 of a matrix whose row 9 couples to rows 0..8
        lrp2, lci2, lval2 = _spd_lower(12, extra_row=9)
        a = lrp2[9]
        swapped = lci2.copy()
        swapped[a], swapped[a + 1] = lci2[a + 1], lci2[a]
        assert _Dev(lrp2, swapped, lval2).call(h.lib, 1.1)[0] == _capi.SSG_ERR_ARG
        good()
        # a row of 33 entries (the kernel takes 32)
        lrp3, lci3, lval3 = _spd_lower(40, extra_row=32)
        assert lrp3[33] - lrp3[32] == 33
        assert _Dev(lrp3, lci3, lval3).call(h.lib, 1.1)[0] == _capi.SSG_ERR_ARG
        good()
    finally:
        h.close()


@pytest.mark.gpu
def test_noalloc_refuses_a_capturing_stream():
    import torch
    from sparsesolv_gb300 import _native
    lrp, lci, lval = _spd_lower(10)
    d = _Dev(lrp, lci, lval)
    lib = _native.load_solver()
    y = torch.zeros(4, device=d.dev)
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream(device=d.dev)
    torch.cuda.synchronize(d.dev)
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            rc = lib.ssg_ic_factor_noalloc(d.n, d.nnz, _ptr(d.lrp), _ptr(d.lci), _ptr(d.val), _ptr(d.out), _ptr(d.D),
                                           1.1, d.vtype, ctypes.c_void_p(s.cuda_stream))
            y.add_(1.0)
    assert rc == _capi.SSG_ERR_STATE
    g.replay()
    torch.cuda.synchronize(d.dev)
    assert float(y[0]) == 1.0
    rc2, _, _ = d.call(lib, 1.1)
    assert rc2 == _capi.SSG_OK
