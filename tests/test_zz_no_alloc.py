"""ssg_ic_factor_noalloc: the IC(0) factor for callers that may not allocate
device memory, checked against the handle's factor (ssg_factor) on the same
matrices, over two calls in a row (the shared scratch must be cleared between
calls). Named to be collected last."""
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


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["real", "complex"])
def test_noalloc_factor_matches_handle_factor(name):
    import torch
    if name == "real":
        rp, ci, val, _ = voxel.config1().assemble()
    else:
        rp, ci, val, _ = voxel.eddy_current_case(6, seed=5).assemble()
    n = len(rp) - 1
    lrp, lci, lval = lower_part(rp, ci, val)
    nnz = len(lci)
    vtype = _capi.COMPLEX if np.iscomplexobj(val) else _capi.REAL
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    d_lrp = torch.from_numpy(lrp).to(dev)
    d_lci = torch.from_numpy(lci).to(dev)
    d_val = torch.from_numpy(lval).to(dev)
    d_out = torch.empty_like(d_val)
    d_D = torch.empty(n, dtype=d_val.dtype, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    h = _capi.Handle(0)
    try:
        h.set_matrix(rp, ci, val)
        for alpha in (1.1, 1.05):  # two calls in a row, the second on the first one's scratch
            ref_lrp, ref_lci, ref_lval, ref_D = h.factor(alpha)
            assert np.array_equal(ref_lrp, lrp) and np.array_equal(ref_lci, lci)
            d_out.fill_(float("nan"))
            d_D.fill_(float("nan"))
            rc = h.lib.ssg_ic_factor_noalloc(n, nnz, _ptr(d_lrp), _ptr(d_lci), _ptr(d_val), _ptr(d_out), _ptr(d_D),
                                             alpha, vtype, stream)
            assert rc == _capi.SSG_OK, rc
            np.testing.assert_allclose(d_out.cpu().numpy(), ref_lval, rtol=1e-12, atol=0)
            np.testing.assert_allclose(d_D.cpu().numpy(), ref_D, rtol=1e-12, atol=0)
        # in place: lval is the input array
        d_in = d_val.clone()
        rc = h.lib.ssg_ic_factor_noalloc(n, nnz, _ptr(d_lrp), _ptr(d_lci), _ptr(d_in), _ptr(d_in), _ptr(d_D), 1.05,
                                         vtype, stream)
        assert rc == _capi.SSG_OK, rc
        np.testing.assert_allclose(d_in.cpu().numpy(), ref_lval, rtol=1e-12, atol=0)
    finally:
        h.close()
