"""Replicas across GPUs: the Krylov path does not shard (IC(0) and its
triangular solves are sequential in natural order), so several GPUs run
independent solves. This module holds the host-side pieces of that: the
assignment of independent systems to ranks and the max-over-ranks timing.
No collective touches the data path; the only collectives are the timing
reduction and barriers between timed regions."""
from __future__ import annotations

import heapq

import numpy as np


def assign_systems(work, world_size):
    """Greedy longest-first assignment of independent systems to ranks.

    ``work[i]`` is the cost estimate of system i (rows, or nonzeros). Returns
    one sorted index list per rank; every system lands on exactly one rank and
    the result depends only on ``work`` and ``world_size``, so every rank
    computes the same assignment without communicating."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    work = np.asarray(work, dtype=np.float64)
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    heap = [(0.0, r) for r in range(world_size)]
    out = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(work[i]), r))
    return [sorted(x) for x in out]


def max_over_ranks(values, group=None):
    """Element-wise maximum of a list of floats over all ranks (identity on
    one process). Used for the timed region: the job ends when the slowest
    rank ends."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return [float(v) for v in values]
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return [float(v) for v in t.cpu()]


def whole_job_rate(units_per_rank, world_size, ms_max):
    """Units per second of the whole job: all ranks' units over the slowest
    rank's time."""
    return float(units_per_rank) * world_size / (ms_max / 1e3)
