"""Batched solves (ssg_batch_*): many systems of uneven sizes and several
right-hand sides in shared launches.

Each instance must match what the reference computes for that system alone
(iteration count within 3% real / 10% complex of the oracle, residual log
within 1e-6 relative, solution within 1e-6 of the oracle's), and its numbers
must be bit-identical whether it is solved alone or inside a batch."""
import numpy as np
import pytest

from oracle.oracle import Settings
from sparsesolv_gb300 import _capi, voxel

pytestmark = pytest.mark.gpu

ALPHA = 1.1


def iter_slack(iters, is_complex):
    return max(2, int((0.10 if is_complex else 0.03) * iters + 0.999))


SIZES = ((6, 1), (9, 2), (12, 3), (7, 4), (10, 5))


def real_systems():
    return [voxel.curl_curl_case(N, seed=seed, iron_size=max(2, N // 3)).assemble() for N, seed in SIZES]


def complex_systems():
    return [voxel.eddy_current_case(N, seed=s).assemble() for N, s in ((5, 3), (7, 4), (6, 9))]


def coil_rhs(k, count, seed):
    """``count`` right-hand sides of system k from seeded coil placements (the
    curl-curl matrix is singular; a coil's divergence-free current keeps the
    system consistent)."""
    N, s0 = SIZES[k]
    case = voxel.curl_curl_case(N, seed=s0, iron_size=max(2, N // 3))
    rng = np.random.default_rng(seed)
    return np.stack([case.rhs([voxel.seeded_coil(rng, N)]) for _ in range(count)])


@pytest.fixture(scope="module")
def systems():
    return real_systems()


def check_against_oracle(oracle, method, rp, ci, va, b, x, log, iters, cplx):
    s = Settings(accel_factor=ALPHA, precondition_type=0)
    ores = oracle.solve(method, rp, ci, va, b, s, conv=1e-8, maxit=5000)
    assert abs(iters - ores.iters) <= iter_slack(ores.iters, cplx), (iters, ores.iters)
    m = min(len(log), len(ores.log))
    if cplx:
        assert np.allclose(log[:3], ores.log[:3], rtol=1e-8)
        import scipy.sparse as sp
        A = sp.csr_matrix((va, ci, rp))
        assert np.linalg.norm(A @ x - A @ ores.x) <= 5e-8 * np.linalg.norm(b)
    else:
        assert np.allclose(log[:m], ores.log[:m], rtol=1e-6, atol=1e-13 * ores.log[0])
        assert np.linalg.norm(x - ores.x) <= 1e-6 * np.linalg.norm(ores.x)


@pytest.mark.parametrize("method", ["iccg", "mrtr"])
def test_real_batch_matches_oracle_per_system(gpu, oracle, systems, method):
    bt = _capi.Batch(0)
    try:
        for rp, ci, va, b in systems:
            bt.add(rp, ci, va, b)
        bt.start(_capi.METHOD_ICCG if method == "iccg" else _capi.METHOD_MRTR, ALPHA, conv=1e-8, max_ite=5000)
        bt.wait()
        for k, (rp, ci, va, b) in enumerate(systems):
            X, it, stt, ok = bt.result(k)
            assert ok and stt[0] == 1
            check_against_oracle(oracle, method, rp, ci, va, b, X[0], bt.residual_log(k), int(it[0]), False)
    finally:
        bt.close()


def test_complex_mrtr_batch_matches_oracle(gpu, oracle):
    bt = _capi.Batch(0)
    cs = complex_systems()
    try:
        for rp, ci, va, b in cs:
            bt.add(rp, ci, va, b)
        bt.start(_capi.METHOD_MRTR, ALPHA, conv=1e-8, max_ite=5000)
        bt.wait()
        for k, (rp, ci, va, b) in enumerate(cs):
            X, it, stt, ok = bt.result(k)
            assert ok
            check_against_oracle(oracle, "mrtr", rp, ci, va, b, X[0], bt.residual_log(k), int(it[0]), True)
    finally:
        bt.close()


def solve_alone(rp, ci, va, B, method):
    bt = _capi.Batch(0)
    try:
        bt.add(rp, ci, va, B)
        bt.start(method, ALPHA, conv=1e-8, max_ite=5000)
        bt.wait()
        X, it, _, _ = bt.result(0)
        logs = [bt.residual_log(0, j) for j in range(len(it))]
        return X, it, logs
    finally:
        bt.close()


@pytest.mark.parametrize("method", [_capi.METHOD_ICCG, _capi.METHOD_MRTR])
def test_instance_identical_alone_and_in_the_mix(gpu, systems, method):
    """Multi-RHS systems in a mix of uneven sizes; each (system, rhs) must give
    bit-identical x, iteration count and residual log when solved alone."""
    Bs = []
    bt = _capi.Batch(0)
    try:
        for k, (rp, ci, va, b) in enumerate(systems):
            B = coil_rhs(k, 1 + k % 3, 100 + k)
            B[0] = b
            Bs.append(B)
            bt.add(rp, ci, va, B)
        bt.start(method, ALPHA, conv=1e-8, max_ite=5000)
        while not bt.poll():  # the non-blocking path
            pass
        mix = [bt.result(k) for k in range(len(systems))]
        mix_logs = [[bt.residual_log(k, j) for j in range(len(Bs[k]))] for k in range(len(systems))]
    finally:
        bt.close()
    for k in (0, 2, 4):
        rp, ci, va, _ = systems[k]
        X, it, logs = solve_alone(rp, ci, va, Bs[k], method)
        assert np.array_equal(X, mix[k][0])
        assert np.array_equal(it, mix[k][1])
        for a, m in zip(logs, mix_logs[k]):
            assert np.array_equal(a, m)


def test_zero_rhs_and_repeated_start(gpu, systems):
    rp, ci, va, b = systems[1]
    B = np.stack([b, np.zeros_like(b)])
    bt = _capi.Batch(0)
    try:
        bt.add(rp, ci, va, B)
        for _ in range(2):  # the second start re-factors and reuses the assembled batch
            bt.start(_capi.METHOD_ICCG, ALPHA, conv=1e-8, max_ite=5000)
            bt.wait()
            X, it, stt, ok = bt.result(0)
            assert ok and it[1] == 0 and np.all(X[1] == 0)
            assert list(bt.residual_log(0, 1)) == [0.0]
            assert it[0] > 5
        # swapped right-hand sides through set_rhs: the results swap with them
        bt.set_rhs(0, B[::-1])
        bt.start(_capi.METHOD_ICCG, ALPHA, conv=1e-8, max_ite=5000)
        bt.wait()
        X2, it2, _, ok2 = bt.result(0)
        assert ok2 and it2[0] == 0 and np.all(X2[0] == 0)
        assert np.array_equal(X2[1], X[0]) and it2[1] == it[0]
    finally:
        bt.close()


def test_batch_argument_errors(gpu, systems):
    rp, ci, va, b = systems[0]
    bt = _capi.Batch(0)
    try:
        with pytest.raises(_capi.SolverError):
            bt.start(_capi.METHOD_ICCG, ALPHA)  # empty batch
        bt.add(rp, ci, va, b)
        with pytest.raises(_capi.SolverError):
            bt.add(rp, ci, va.astype(np.complex128), b)  # mixed real / complex
        with pytest.raises(_capi.SolverError):
            bt.start(_capi.METHOD_ICCG, -1.0)  # no automatic shift in batches
    finally:
        bt.close()


def test_finished_system_result_while_batch_runs(gpu):
    """A small system's result can be taken as soon as it ends; it equals the
    result read after the whole batch ended."""
    small = voxel.curl_curl_case(6, seed=1, iron_size=2).assemble()
    large = voxel.curl_curl_case(24, seed=2, iron_size=6).assemble()
    bt = _capi.Batch(0)
    try:
        bt.add(*small)
        bt.add(*large)
        bt.start(_capi.METHOD_ICCG, ALPHA, conv=1e-8, max_ite=5000)
        early = None
        done = False
        while not done:
            done = bt.step()
            if early is None and bt.finished(0):
                early = bt.result(0)
                seen_running = not done
        assert early is not None and seen_running
        late = bt.result(0)
        assert np.array_equal(early[0], late[0]) and np.array_equal(early[1], late[1])
        with pytest.raises(_capi.SolverError):  # a running system's result is refused
            bt.start(_capi.METHOD_ICCG, ALPHA, conv=1e-8, max_ite=5000)
            try:
                if not bt.finished(1):
                    bt.result(1)
                else:
                    raise _capi.SolverError(-6, "large system ended before the check")
            finally:
                bt.wait()
    finally:
        bt.close()


@pytest.mark.parametrize("precision", [_capi.PREC_FP64, _capi.PREC_MIXED])
def test_graph_replay_equals_direct_launches(gpu, systems, precision):
    """Chunks replayed from a captured CUDA graph give the same bits as direct launches."""
    out = {}
    for graphs in (True, False):
        bt = _capi.Batch(0)
        try:
            bt.set_graphs(graphs)
            bt.set_precision(precision)
            for rp, ci, va, b in systems:
                bt.add(rp, ci, va, b)
            l0 = bt.lib.ssg_launch_count()
            bt.start(_capi.METHOD_ICCG, ALPHA, conv=1e-8, max_ite=5000)
            bt.wait()
            out[graphs] = [bt.result(k) for k in range(len(systems))], bt.lib.ssg_launch_count() - l0
        finally:
            bt.close()
    for a, b in zip(out[True][0], out[False][0]):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    # replayed kernels are counted too: the same iterations, a similar count (no-op tail launches differ)
    assert out[True][1] > 0.5 * out[False][1]


def test_autotuned_batch_meets_the_bar_and_stays_deterministic(gpu, oracle, systems):
    """ssg_batch_autotune picks a sweep schedule by timing; the batch then still
    matches the oracle per system, and repeated starts give the same bits."""
    bt = _capi.Batch(0)
    try:
        for k, (rp, ci, va, b) in enumerate(systems):
            bt.add(rp, ci, va, coil_rhs(k, 2, seed=40 + k) if k == 1 else b)
        c = bt.autotune()
        assert c["mode"] in (1, 2, 3) and c["group"] in (4, 8, 16) and c["ms"] > 0
        runs = []
        for _ in range(2):
            bt.start(_capi.METHOD_ICCG, ALPHA, conv=1e-8, max_ite=5000)
            bt.wait()
            runs.append([bt.result(k) for k in range(len(systems))])
        for k, (rp, ci, va, b) in enumerate(systems):
            X, it, stt, ok = runs[0][k]
            assert ok and np.array_equal(X, runs[1][k][0]) and np.array_equal(it, runs[1][k][1])
            if k != 1:
                check_against_oracle(oracle, "iccg", rp, ci, va, b, X[0], bt.residual_log(k), int(it[0]), False)
    finally:
        bt.close()


def _persist_run(persist, systems, Bs):
    bt = _capi.Batch(0)
    try:
        bt.set_persistent(persist)
        for (rp, ci, va, _), B in zip(systems, Bs):
            bt.add(rp, ci, va, B)
        bt.start(_capi.METHOD_ICCG, ALPHA, conv=1e-8, max_ite=5000)
        bt.wait()
        res = [bt.result(k) for k in range(len(systems))]
        logs = [[bt.residual_log(k, j) for j in range(len(Bs[k]))] for k in range(len(systems))]
        return res, logs
    finally:
        bt.close()


def test_persistent_batch_same_bits_as_launches(gpu, oracle):
    """ssg_batch_set_persistent: one CTA per instance runs all of its iterations. Every
    instance gives the same bits as the launch-per-phase iterations (x, iteration
    count, residual log) and meets the oracle. A batch holding a system of more than
    16,384 rows runs the launches (same bits again)."""
    rng = np.random.default_rng(17)
    systems = [voxel.curl_curl_case(N, seed=30 + N, iron_size=max(2, N // 3)).assemble() for N in (6, 8, 10, 12)]
    import scipy.sparse as sp
    Bs = []
    for rp, ci, va, b in systems:
        A = sp.csr_matrix((va, ci, rp))
        Bs.append(np.stack([b, A @ rng.standard_normal(len(b))]))  # a consistent second right-hand side
    ref, ref_logs = _persist_run(False, systems, Bs)
    got, got_logs = _persist_run(True, systems, Bs)  # the default
    for k in range(len(systems)):
        assert np.array_equal(got[k][0], ref[k][0]) and np.array_equal(got[k][1], ref[k][1]), k
        for a, m in zip(got_logs[k], ref_logs[k]):
            assert np.array_equal(a, m)
        rp, ci, va, b = systems[k]
        check_against_oracle(oracle, "iccg", rp, ci, va, b, got[k][0][0], got_logs[k][0], int(got[k][1][0]), False)
    # with a 20^3 system (21,660 rows) in the batch: the launches run
    big = voxel.config1().assemble()
    systems2 = systems[:2] + [big]
    Bs2 = Bs[:2] + [np.atleast_2d(big[3])]
    ref2, _ = _persist_run(False, systems2, Bs2)
    got2, _ = _persist_run(True, systems2, Bs2)
    for k in range(3):
        assert np.array_equal(got2[k][0], ref2[k][0]) and np.array_equal(got2[k][1], ref2[k][1])
