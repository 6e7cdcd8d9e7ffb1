"""Serving loop: solve requests that arrive over time, with continuous batching.

Requests of one kind (real ICCG, complex IC-MRTR) wait in that kind's queue.
Each kind has a few slots; a slot is a reusable batch (its own CUDA stream,
device buffers kept between uses and between streams) served by one worker
thread. A free slot takes the waiting requests of its kind in arrival order
(optionally only those of similar size), as many as fit its row budget and
the free device memory, solves them in shared launches and hands each result
back as soon as that request's own solve has ended. A batch costs about the
depth x iterations of its largest system, so smaller systems ride along
nearly free, and early delivery keeps their latency their own. Requests that arrive while others are on the GPU are
admitted by the next slot that frees up, so the work of several batches
overlaps on the device (the C calls release the GIL).

Every instance's numbers are independent of the batch it lands in (the
batched kernels reduce per instance in a fixed order), so a request's result
is the same alone and in the mix.
"""
from __future__ import annotations

import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

KIND_REAL_ICCG = "real-iccg"
KIND_COMPLEX_MRTR = "complex-mrtr"


@dataclass
class Request:
    rid: int
    arrival: float       # seconds after the stream starts
    row_ptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    b: np.ndarray
    kind: str = KIND_REAL_ICCG
    # filled in by the server
    admitted: float = -1.0
    done: float = -1.0
    x: np.ndarray = None
    iters: int = -1
    converged: bool = False
    batch_size: int = 0

    @property
    def n(self):
        return len(self.row_ptr) - 1

    @property
    def nnz(self):
        return len(self.col)

    @property
    def latency(self):
        return self.done - self.arrival


class GpuBackend:
    """Slots are ssg_batch objects; free memory from the CUDA runtime.

    precision None picks per kind, by measurement: real curl-curl ICCG in mixed
    precision (two refinement steps, faster at every size), complex
    eddy-current IC-MRTR in FP64 (FP32 rounding of these systems lets one inner
    solve gain little, so large ones need dozens of refinement steps and run
    slower than FP64)."""

    def __init__(self, device=0, precision=None, alpha=1.1, tol=1e-8, max_ite=5000):
        from . import _capi
        self.capi = _capi
        self.device = device
        self.precision = precision
        self.alpha, self.tol, self.max_ite = alpha, tol, max_ite

    def precision_of(self, kind):
        if self.precision is not None:
            return self.precision
        return self.capi.PREC_MIXED if kind == KIND_REAL_ICCG else self.capi.PREC_FP64

    def new_slot(self, kind):
        bt = self.capi.Batch(self.device)
        bt.set_precision(self.precision_of(kind))
        return bt

    def free_bytes(self):
        import torch
        free, _ = torch.cuda.mem_get_info(self.device)
        return int(free)

    def solve(self, slot, kind, reqs, deliver=None):
        """Blocking: solve reqs in one batch on slot; fills x, iters, converged
        and calls deliver(r) for each request as soon as its own solve ended."""
        slot.clear()
        for r in reqs:
            slot.add(r.row_ptr, r.col, r.val, r.b)
        meth = self.capi.METHOD_ICCG if kind == KIND_REAL_ICCG else self.capi.METHOD_MRTR
        slot.start(meth, self.alpha, conv=self.tol, max_ite=self.max_ite)
        pending = list(range(len(reqs)))
        while pending:
            done = slot.step()
            for k in [k for k in pending if done or slot.finished(k)]:
                X, it, _, ok = slot.result(k)
                r = reqs[k]
                r.x, r.iters, r.converged = X[0], int(it[0]), bool(ok)
                pending.remove(k)
                if deliver:
                    deliver(r)

    def close_slot(self, slot):
        slot.close()


@dataclass
class ServerConfig:
    slots: dict = field(default_factory=lambda: {KIND_REAL_ICCG: 3, KIND_COMPLEX_MRTR: 2})
    max_rows_per_batch: int = 3_000_000
    size_ratio: float = 0.0            # > 1: a batch only groups requests within this factor of its oldest one
    share: bool = False                # a batch takes at most the waiting rows / the kind's slots (spreads the
                                       # work of a burst over the slots, which then run side by side)
    bytes_per_nnz: float = 96.0        # device bytes a request needs per matrix entry (estimate)
    memory_reserve: int = 2 << 30      # left free for everything else


class Server:
    def __init__(self, backend, config=None, clock=time.perf_counter):
        self.backend = backend
        self.cfg = config or ServerConfig()
        self.clock = clock
        self.lock = threading.Condition()
        self.queues = {k: deque() for k in self.cfg.slots}
        self.reserved = 0          # bytes promised to batches being set up or solved
        self.t0 = None
        self.closed = False
        self.errors = []
        self.workers = []
        self._slots = {}           # (kind, index) -> backend slot, kept across runs

    # -- admission
    def _need(self, r):
        return int(r.nnz * self.cfg.bytes_per_nnz)

    def _take(self, kind):
        """Called with the lock held: the next batch for a slot of this kind.
        It starts with the oldest waiting request and adds, in arrival order,
        waiting requests within ``size_ratio`` of its size (similar depth and
        iteration count, so no instance idles behind a much longer one), within
        the row budget and the free memory."""
        q = self.queues[kind]
        if not q:
            return []
        free = self.backend.free_bytes() - self.cfg.memory_reserve - self.reserved
        head = q[0]
        if self._need(head) > free and self.reserved > 0:
            return []  # wait for memory held by running batches
        out, rows, need = [head], head.n, self._need(head)
        budget = self.cfg.max_rows_per_batch
        if self.cfg.share:
            budget = min(budget, max(head.n, sum(r.n for r in q) // max(1, self.cfg.slots[kind])))
        ratio = self.cfg.size_ratio if self.cfg.size_ratio > 1.0 else float("inf")
        lo, hi = head.n / ratio, head.n * ratio
        for r in list(q)[1:]:
            if not lo <= r.n <= hi:
                continue
            nr = self._need(r)
            if rows + r.n > budget or need + nr > free:
                break
            out.append(r)
            rows += r.n
            need += nr
        taken = {id(r) for r in out}
        self.queues[kind] = deque(r for r in q if id(r) not in taken)
        self.reserved += need
        return out

    def _slot(self, kind, index):
        key = (kind, index)
        if key not in self._slots:
            self._slots[key] = self.backend.new_slot(kind)
        return self._slots[key]

    def close(self):
        for slot in self._slots.values():
            self.backend.close_slot(slot)
        self._slots = {}

    def _worker(self, kind, index):
        slot = self._slot(kind, index)
        while True:
            with self.lock:
                while True:
                    reqs = self._take(kind)
                    if reqs or (self.closed and not self.queues[kind]):
                        break
                    self.lock.wait(0.05)
            if not reqs:
                return
            now = self.clock() - self.t0
            for r in reqs:
                r.admitted = now
                r.batch_size = len(reqs)

            def deliver(r):
                r.done = self.clock() - self.t0

            try:
                self.backend.solve(slot, kind, reqs, deliver)
            except Exception as e:  # recorded; the requests stay unsolved
                self.errors.append(e)
            done = self.clock() - self.t0
            with self.lock:
                for r in reqs:
                    if r.done < 0:
                        r.done = done
                self.reserved -= sum(self._need(r) for r in reqs)
                self.lock.notify_all()

    # -- driving a request stream in real time
    def run(self, requests):
        """Feed requests at their arrival times; return when all are done."""
        reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
        for r in reqs:
            if r.kind not in self.queues:
                raise ValueError("no slots for request kind %r" % r.kind)
        self.t0 = self.clock()
        self.closed = False
        self.workers = [threading.Thread(target=self._worker, args=(k, i), daemon=True)
                        for k, count in self.cfg.slots.items() for i in range(count)]
        for w in self.workers:
            w.start()
        for r in reqs:
            delay = r.arrival - (self.clock() - self.t0)
            if delay > 0:
                time.sleep(delay)
            with self.lock:
                self.queues[r.kind].append(r)
                self.lock.notify_all()
        with self.lock:
            self.closed = True
            self.lock.notify_all()
        for w in self.workers:
            w.join()
        if self.errors:
            raise self.errors[0]
        return reqs


def latency_stats(reqs):
    lat = np.array([r.latency for r in reqs])
    span = max(r.done for r in reqs) - min(r.arrival for r in reqs)
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "solves_per_s": len(reqs) / span if span > 0 else float("inf"),
            "requests": len(reqs), "mean_batch": float(np.mean([r.batch_size for r in reqs]))}


def synthetic_stream(count, rate, seed=5, lo=1_000, hi=500_000, complex_share=0.3):
    """Poisson arrivals at ``rate`` requests/s (rate <= 0: all at t = 0), sizes
    log-uniform in [lo, hi] unknowns, 70% real curl-curl (ICCG) and 30%
    complex eddy-current (IC-MRTR) systems from the seeded voxel generator."""
    from . import voxel
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        if rate > 0:
            t += rng.exponential(1.0 / rate)
        target = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        # n = 3 N (N - 1)^2 unknowns for an N^3 voxel cube
        N = max(6, int(round((target / 3.0) ** (1.0 / 3.0))) + 1)
        sub = int(rng.integers(0, 2**31 - 1))
        if rng.uniform() < complex_share:
            rp, ci, va, b = voxel.eddy_current_case(N, seed=sub).assemble()
            kind = KIND_COMPLEX_MRTR
        else:
            rp, ci, va, b = voxel.curl_curl_case(N, seed=sub, n_iron=1, iron_size=max(2, N // 4)).assemble()
            kind = KIND_REAL_ICCG
        out.append(Request(i, t if rate > 0 else 0.0, rp, ci, va, b, kind))
    return out
