"""Serving-loop scheduling on the CPU with a fake batch backend: every request
completes, batches hold one kind and start with the oldest waiting request
(grouping requests of similar size), the row budget and the free-memory limit hold, and requests that arrive while batches
run are admitted before those batches finish (continuous batching)."""
from __future__ import annotations

import threading
import time

import numpy as np

from sparsesolv_gb300 import serving
from sparsesolv_gb300.serving import KIND_COMPLEX_MRTR, KIND_REAL_ICCG, Request, Server, ServerConfig


class FakeBackend:
    def __init__(self, free=1 << 40, sec_per_row=2e-6):
        self.free = free
        self.sec_per_row = sec_per_row
        self.batches = []
        self.lock = threading.Lock()
        self.active = 0
        self.max_active = 0

    def new_slot(self, kind):
        return object()

    def close_slot(self, slot):
        pass

    def free_bytes(self):
        return self.free

    def solve(self, slot, kind, reqs, deliver=None):
        with self.lock:
            self.batches.append((kind, [r.rid for r in reqs]))
            self.active += 1
            self.max_active = max(self.max_active, self.active)
        time.sleep(self.sec_per_row * sum(r.n for r in reqs))
        for r in reqs:
            r.x = np.full(r.n, float(r.rid))
            r.iters, r.converged = 1, True
            if deliver:
                deliver(r)
        with self.lock:
            self.active -= 1


def req(rid, arrival, n, kind=KIND_REAL_ICCG, nnz_per_row=33):
    rp = np.arange(n + 1, dtype=np.int32) * nnz_per_row
    return Request(rid, arrival, rp, np.zeros(n * nnz_per_row, np.int32), np.zeros(n * nnz_per_row),
                   np.ones(n), kind)


def test_all_requests_complete_in_kind_and_arrival_order():
    be = FakeBackend()
    cfg = ServerConfig(slots={KIND_REAL_ICCG: 2, KIND_COMPLEX_MRTR: 1}, max_rows_per_batch=50_000, memory_reserve=0,
                       size_ratio=2.0)
    rng = np.random.default_rng(0)
    reqs = [req(i, 0.002 * i, int(rng.integers(1_000, 20_000)),
                KIND_COMPLEX_MRTR if i % 3 == 0 else KIND_REAL_ICCG) for i in range(40)]
    out = Server(be, cfg).run(reqs)
    assert all(r.converged and r.done >= r.admitted >= r.arrival for r in out)
    assert all(np.all(r.x == r.rid) for r in out)
    kinds = {r.rid: r.kind for r in reqs}
    for kind, ids in be.batches:
        assert all(kinds[i] == kind for i in ids)
        assert len(ids) == 1 or sum(reqs[i].n for i in ids) <= cfg.max_rows_per_batch
    for kind in (KIND_REAL_ICCG, KIND_COMPLEX_MRTR):
        mine = [ids for k, ids in be.batches if k == kind]
        heads = [ids[0] for ids in mine]
        assert heads == sorted(heads)  # every batch starts with the oldest waiting request
        for ids in mine:  # and groups requests of similar size with it, in arrival order
            assert ids == sorted(ids)
            assert all(reqs[ids[0]].n / cfg.size_ratio <= reqs[i].n <= reqs[ids[0]].n * cfg.size_ratio for i in ids)
        assert sorted(i for ids in mine for i in ids) == [r.rid for r in reqs if r.kind == kind]


def test_default_batches_fill_in_arrival_order():
    be = FakeBackend()
    cfg = ServerConfig(slots={KIND_REAL_ICCG: 1}, max_rows_per_batch=25_000, memory_reserve=0)
    rng = np.random.default_rng(1)
    reqs = [req(i, 0.0, int(rng.integers(1_000, 20_000))) for i in range(20)]
    Server(be, cfg).run(reqs)
    order = [i for _, ids in be.batches for i in ids]
    assert order == list(range(20))  # one slot: batches are consecutive runs of the queue
    for _, ids in be.batches:
        assert len(ids) == 1 or sum(reqs[i].n for i in ids) <= cfg.max_rows_per_batch


def test_free_memory_limits_admission():
    n = 5_000
    cfg = ServerConfig(slots={KIND_REAL_ICCG: 3}, max_rows_per_batch=10**9, bytes_per_nnz=100.0, memory_reserve=0)
    need = int(n * 33 * cfg.bytes_per_nnz)
    be = FakeBackend(free=2 * need + 1)
    out = Server(be, cfg).run([req(i, 0.0, n) for i in range(12)])
    assert all(r.converged for r in out)
    # never more than two requests' worth of memory promised at once
    assert max(len(ids) for _, ids in be.batches) <= 2


def test_late_arrivals_are_admitted_while_earlier_batches_run():
    be = FakeBackend(sec_per_row=2e-5)
    cfg = ServerConfig(slots={KIND_REAL_ICCG: 3}, max_rows_per_batch=10_000, memory_reserve=0)
    reqs = [req(0, 0.0, 10_000), req(1, 0.02, 2_000), req(2, 0.04, 2_000)]
    out = Server(be, cfg).run(reqs)
    first = out[0]
    assert out[1].admitted < first.done and out[2].admitted < first.done
    assert be.max_active >= 2


def test_latency_stats_and_stream_shape():
    reqs = [req(i, 0.1 * i, 1_000) for i in range(5)]
    for k, r in enumerate(reqs):
        r.admitted, r.done, r.batch_size = r.arrival, r.arrival + 0.01 * (k + 1), 1
    st = serving.latency_stats(reqs)
    assert abs(st["p50_ms"] - 30.0) < 1e-6 and st["requests"] == 5
    s = serving.synthetic_stream(6, rate=100.0, seed=1, lo=1_000, hi=3_000)
    assert len(s) == 6 and all(s[i].arrival <= s[i + 1].arrival for i in range(5))
    assert all(1_000 // 2 <= r.n <= 3 * 3_000 for r in s)
    assert {r.kind for r in s} <= {KIND_REAL_ICCG, KIND_COMPLEX_MRTR}


def test_share_spreads_a_burst_over_the_slots():
    be = FakeBackend(sec_per_row=1e-6)
    cfg = ServerConfig(slots={KIND_REAL_ICCG: 4}, max_rows_per_batch=10**9, memory_reserve=0, share=True)
    reqs = [req(i, 0.0, 5_000) for i in range(16)]
    out = Server(be, cfg).run(reqs)
    assert all(r.converged for r in out)
    # the first batch takes a quarter of the burst, not all of it
    assert len(be.batches[0][1]) == 4
    assert be.max_active >= 2
    assert sorted(i for _, ids in be.batches for i in ids) == list(range(16))
