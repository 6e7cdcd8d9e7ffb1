"""Serving loop on the GPU: a stream of real ICCG and complex IC-MRTR requests
of uneven sizes, admitted into concurrent batches as they arrive (mixed
precision to 1e-8). Each result must reach the tolerance on the true residual
and be bit-identical to the same request solved alone."""
import numpy as np
import pytest
import scipy.sparse as sp

from sparsesolv_gb300 import _capi, serving

pytestmark = pytest.mark.gpu


def test_stream_results_match_alone(gpu):
    reqs = serving.synthetic_stream(12, rate=300.0, seed=7, lo=1_000, hi=30_000)
    be = serving.GpuBackend(0)
    cfg = serving.ServerConfig(slots={serving.KIND_REAL_ICCG: 2, serving.KIND_COMPLEX_MRTR: 2},
                               max_rows_per_batch=60_000)
    srv = serving.Server(be, cfg)
    try:
        out = srv.run(reqs)
    finally:
        srv.close()
    assert any(r.batch_size > 1 for r in out), "no request shared a batch"
    for r in out:
        assert r.converged
        A = sp.csr_matrix((r.val, r.col, r.row_ptr))
        assert np.linalg.norm(r.b - A @ r.x) <= 1e-8 * np.linalg.norm(r.b)
    # alone: a batch of one on a fresh slot
    for r in out:
        slot = be.new_slot(r.kind)
        try:
            alone = serving.Request(r.rid, 0.0, r.row_ptr, r.col, r.val, r.b, r.kind)
            be.solve(slot, r.kind, [alone])
        finally:
            be.close_slot(slot)
        assert np.array_equal(alone.x, r.x) and alone.iters == r.iters
