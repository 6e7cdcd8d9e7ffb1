"""Host logic of the multi-GPU replicas (no GPU): the system assignment and the
max-over-ranks timing, run as two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from sparsesolv_gb300 import replicas


def test_assignment_covers_every_system_once_and_balances():
    rng = np.random.default_rng(0)
    work = rng.integers(1_000, 100_000, size=257)
    for ws in (1, 2, 3, 8):
        parts = replicas.assign_systems(work, ws)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(work)))
        loads = [work[p].sum() for p in parts]
        assert max(loads) - min(loads) <= work.max()  # greedy longest-first bound
    assert replicas.assign_systems([], 4) == [[], [], [], []]
    with pytest.raises(ValueError):
        replicas.assign_systems([1, 2], 0)


def test_whole_job_rate():
    assert replicas.whole_job_rate(3, 2, 1500.0) == pytest.approx(4.0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world_size, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        work = np.arange(1, 41) * 997 % 101 + 1
        mine = replicas.assign_systems(work, world_size)[rank]
        local_ms = [10.0 * (rank + 1), 5.0 - rank]
        mx = replicas.max_over_ranks(local_ms)
        np.save(os.path.join(out_dir, "r%d.npy" % rank), np.array(mx + [len(mine)] + mine, dtype=np.float64))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r0 = np.load(tmp_path / "r0.npy")
    r1 = np.load(tmp_path / "r1.npy")
    assert list(r0[:2]) == [20.0, 5.0] and list(r1[:2]) == [20.0, 5.0]
    s0 = set(r0[3:3 + int(r0[2])].astype(int))
    s1 = set(r1[3:3 + int(r1[2])].astype(int))
    assert not (s0 & s1) and (s0 | s1) == set(range(40))
