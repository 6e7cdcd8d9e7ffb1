"""Benchmark of the GB300 Krylov hot path (one JSON line on stdout).

Workload (default): the 80^3-voxel static-magnetic curl-curl system with three
seeded iron blocks (n = 1,497,840 edge unknowns, 48.45M nonzeros, FP64),
solved by shifted ICCG with alpha = 1.1 to relative residual 1e-8 from x = 0.
One step = one solve() as the reference defines it: the IC(0) factorisation
is recomputed every step (new values are pushed through the values-only
update, which keeps only the pattern analysis), then the iterations run to
tolerance. ``value`` is solves per second over the whole job with the matrix
and b resident in HBM; ``e2e`` is the same through the C ABI with host
buffers (values, b and x0 copied in, x copied out inside the timed region).
The line also carries, for the same matrix on the same GPU: the solution's
distance from a full FP64 solve of the oracle (``parity``), the mixed-precision
solve against this plain FP64 one (``mixed``), the serving stream against the
plain path one request at a time (``serving``), the first solve of a new
sparsity pattern (``new_pattern``), and the 256-system batch of the cfg4
workload in FP64 and mixed precision (``batch``).

    python bench.py [--steps K] [--warmup W] [--method iccg|sgs|mrtr_ic]
                    [--workload cfg2|cfg1|cfg3|cfg4|cfg5] [--sweep-mode 0..4]
                    [--impl reference]

Under torchrun (--gpus N > 1) every rank solves its own replica (the path
does not shard; "replicas only") and value sums the ranks' solves.
--impl reference times the reference algorithm on the host cores and touches
no GPU: every step is one full solve to tolerance (factorisation plus every
iteration), by the reference built from its sources (oracle/_ref) where that
build exists, else by the oracle's C restatement of it, with the SpMV on all
host cores as the reference's OpenMP build runs it; one more solve on one
thread is reported beside it.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "time-to-1e-8 residual (s), solves/s, p50/p99 latency vs plain FP64 GPU ICCG"
TOL = 1e-8
ALPHA = 1.1
MAXIT = 20000


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant kernel, from one ncu
# capture of the same workload: profiles/k_sweep_push_80cube.md (push sweeps, the automatic mode's choice for
# real values), profiles/k_sweep_cluster_80cube.md (lockstep cluster sweeps) and profiles/k_sweep_fwd_80cube.md
# (sync-free forward sweep)
NCU_TRAFFIC = {
    ("cfg2", "fp64", "push", "forward sweep"): 434.4e6,
    ("cfg2", "fp64", "push", "backward sweep"): 434.3e6,
    ("cfg2", "fp64", "cluster", "forward sweep"): 348.7e6,
    ("cfg2", "fp64", "cluster", "backward sweep"): 347.6e6,
    ("cfg2", "fp64", "sync-free", "forward sweep"): 360.6e6,
}
# the same captures' FP64 pipe (sm__inst_executed_pipe_fp64, % of peak sustained on the active SMs, averaged over
# all 152): the push sweep runs level by level on one 16-SM cluster, bound by FP64 latency and issue on those SMs
NCU_FP64_PIPE = {
    ("cfg2", "fp64", "push", "forward sweep"): 0.237,
    ("cfg2", "fp64", "push", "backward sweep"): 0.245,
}


def sweep_kind(mode, cplx):
    """The sweep schedule a mode runs: the automatic mode (0) takes the push sweep for real values and the
    one-cluster lockstep sweep for complex ones, where their plans fit."""
    if mode == 0:
        return "cluster" if cplx else "push"
    return {1: "sync-free", 2: "cluster", 3: "neighbour", 4: "push"}.get(mode, "cluster")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--method", default="iccg", choices=["iccg", "sgs", "mrtr_ic"])
    ap.add_argument("--alpha", type=float, default=1.1, help="acceleration factor (shift) of the IC(0) factor")
    ap.add_argument("--workload", default="cfg2", choices=["cfg2", "cfg1", "cfg3", "cfg4", "cfg5"])
    ap.add_argument("--rhs", type=int, default=1,
                    help="cfg2/cfg3: right-hand sides per step, solved in one ssg_solve_multi call "
                         "(the first is the workload's b, the others consistent ones of the same norm)")
    ap.add_argument("--requests", type=int, default=32, help="cfg5: requests per stream")
    ap.add_argument("--slots", default="4,4", help="cfg5: slots for real ICCG, complex IC-MRTR")
    ap.add_argument("--share", action=argparse.BooleanOptionalAction, default=True,
                    help="cfg5: spread a burst's rows over the slots of a kind")
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed"],
                    help="mixed: FP32 inner solves inside FP64 refinement on the true residual "
                         "(default: mixed for the serving stream, fp64 otherwise)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="leave the mixed-precision comparison out of the line")
    ap.add_argument("--no-serving", action="store_true", help="leave the serving stream out of the line")
    ap.add_argument("--no-batch", action="store_true", help="leave the 256-system batch out of the line")
    ap.add_argument("--cpu-threads", type=int, default=0,
                    help="OpenMP threads of the CPU path (reference arm and cpu_baseline); 0: all host cores")
    ap.add_argument("--autotune", action="store_true",
                    help="time the sweep schedules on the workload first (ssg_autotune) and keep the fastest")
    ap.add_argument("--batch-group", type=int, default=0, choices=[0, 4, 8, 16],
                    help="lanes a row in the sweeps of the handle's internal batch (mixed precision, --rhs); 0 auto")
    ap.add_argument("--batch-sizes", default="8,32",
                    help="cfg4: the range of N (voxels a side) of the 256 systems, N ~ U{lo..hi}")
    ap.add_argument("--batch-persistent", action=argparse.BooleanOptionalAction, default=True,
                    help="cfg4: FP64 ICCG starts with one CTA per instance running all its iterations where every "
                         "instance is small enough (the default); --no-batch-persistent: launches per phase")
    ap.add_argument("--sweep-mode", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="triangular sweeps: 0 automatic, 1 sync-free, 2 one-cluster level-synchronous, "
                         "3 one-cluster neighbour-synchronised, 4 one-cluster push")
    return ap.parse_args()


def workload(name):
    from sparsesolv_gb300 import voxel
    if name == "cfg2":
        case, label = voxel.config2(), "curl-curl 80^3 voxels, 3 seeded iron blocks"
    elif name == "cfg3":
        case, label = voxel.config3(), "eddy-current K + j omega sigma M, 60^3 voxels, complex128"
    else:
        case, label = voxel.config1(), "curl-curl 20^3 voxels, 1 seeded iron block"
    t0 = time.perf_counter()
    rp, ci, val, b = case.assemble()
    WORKLOAD_CASE[name] = (case, time.perf_counter() - t0)
    return label, rp, ci, val, b


WORKLOAD_CASE = {}  # workload name -> (voxel case, seconds of its host assembly)


def device_assembly(device, name, rp, ci, val, b):
    """The same system assembled on the GPU (ssg_set_matrix_voxel) on a fresh handle: seconds (host maps and
    element matrices, upload, assembly, scan), against the host generator's seconds, and whether pattern,
    values and right-hand side are bit-identical to the host's."""
    from sparsesolv_gb300 import _capi
    case, t_host = WORKLOAD_CASE[name]
    h = _capi.Handle(device)
    try:
        h.set_matrix_voxel(case)  # first call: the kernels' load
        t0 = time.perf_counter()
        bd = h.set_matrix_voxel(case)
        t_dev = time.perf_counter() - t0
        drp, dci, dva = h.get_matrix()
        same = (np.array_equal(drp, rp) and np.array_equal(dci, ci) and
                np.array_equal(dva.view(np.float64), np.asarray(val).view(np.float64)) and
                np.array_equal(np.asarray(bd).view(np.float64), np.asarray(b).view(np.float64)))
    finally:
        h.close()
    return {"host_generator_s": t_host, "device_s": t_dev, "speedup": t_host / t_dev, "bit_identical": bool(same),
            "what": "the workload's matrix and right-hand side: host C generator (voxelgen.c) vs "
                    "ssg_set_matrix_voxel into a handle (edge maps and element matrices from the host)"}


def method_args(m):
    from sparsesolv_gb300 import _capi
    if m == "iccg":
        return _capi.METHOD_ICCG, 1, "shifted ICCG"
    if m == "sgs":
        return _capi.METHOD_MRTR, 1, "Eisenstat SGS-MRTR"
    return _capi.METHOD_MRTR, 0, "shifted IC-MRTR"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for name, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def host_info():
    """Host cores and CPU model of the machine the CPU path runs on."""
    model = None
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
                             timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"nproc": os.cpu_count(), "cpu_model": model or platform.processor() or platform.machine(),
            "machine": platform.machine()}


def workload_config(label, n, nnz, mname, precision, K):
    """The workload as both arms name it (the same dict in both lines)."""
    return {"workload": label, "n": n, "nnz": nnz, "method": mname, "alpha": ALPHA, "tolerance": TOL,
            "precision": precision, "right_hand_sides": K, "x0": "zero", "factor": "recomputed every step",
            "l2": "inputs larger than L2 (matrix %.0f MB)" % ((12.0 * nnz) / 1e6)}


def extra_rhs(rp, ci, val, b, K):
    """b followed by K - 1 right-hand sides in the range of A (the curl-curl
    systems are singular), each of the norm of b, seeded."""
    if K <= 1:
        return [b]
    n = len(b)
    cplx = np.iscomplexobj(val)
    rng = np.random.default_rng(2024)
    out = [b]
    for _ in range(K - 1):
        v = rng.standard_normal(n) + (1j * rng.standard_normal(n) if cplx else 0.0)
        e = _spmv_host(rp, ci, val, v)
        out.append(e * (np.linalg.norm(b) / np.linalg.norm(e)))
    return out


class CpuPath:
    """The reference algorithm on the host cores: the reference built from its
    sources (oracle/_ref) where that build exists, else the oracle's C
    restatement. Both run the SpMV row-parallel on OpenMP threads, as the
    reference's Eigen product does; the factorisation, sweeps and vector work
    are serial, as in the reference."""

    def __init__(self, method, pt):
        from oracle.oracle import Oracle, Reference, Settings, build
        build()
        self.orc = Oracle()
        self.use_ref = Reference.available()
        self.eng = Reference() if self.use_ref else self.orc
        self.kind = "reference" if self.use_ref else "port"
        self.m = "iccg" if method == "iccg" else "mrtr"
        self.settings = Settings(accel_factor=ALPHA, precondition_type=pt, is_save_residual_log=True)

    def solve(self, rp, ci, val, b, threads):
        """One full solve to tolerance: (result, total s, set-up s or None)."""
        self.orc.set_threads(threads)  # the OpenMP runtime is shared with the reference build
        t0 = time.perf_counter()
        res = self.eng.solve(self.m, rp, ci, val, b, self.settings, conv=TOL, maxit=MAXIT)
        total = time.perf_counter() - t0
        setup = self.orc.last_timings()[0] if not self.use_ref else None
        return res, total, setup

    def setup_seconds(self, rp, ci, val, b, threads):
        """Set-up alone (scaling, factor, transpose): a solve stopped before its
        first iteration (its "not converged" message kept off stdout, which
        carries the JSON line)."""
        self.orc.set_threads(threads)
        sys.stdout.flush()
        saved = os.dup(1)
        devnull = os.open(os.devnull, os.O_WRONLY)
        os.dup2(devnull, 1)
        try:
            t0 = time.perf_counter()
            self.eng.solve(self.m, rp, ci, val, b, self.settings, conv=TOL, maxit=0)
            return time.perf_counter() - t0
        finally:
            os.dup2(saved, 1)
            os.close(saved)
            os.close(devnull)


def phases(res, total, setup):
    it = max(int(res.iters), 1)
    return {"total_s": total, "setup_s": setup, "per_iteration_s": (total - setup) / it if setup is not None else None,
            "iterations": int(res.iters), "converged": bool(res.converged)}


def run_reference(args):
    """The reference's CPU path on the host cores, full solves; no GPU is touched."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    if args.workload not in ("cfg1", "cfg2", "cfg3"):
        print(json.dumps({"impl": "reference", "unavailable": "the CPU arm times single-system workloads "
                          "(cfg1, cfg2, cfg3); %s has no reference counterpart to time" % args.workload}),
              flush=True)
        return
    label, rp, ci, val, b = workload(args.workload)
    _, pt, mname = method_args(args.method)
    n, nnz = len(rp) - 1, len(ci)
    K = max(1, args.rhs)
    bs = extra_rhs(rp, ci, val, b, K)
    cpu = CpuPath(args.method, pt)
    threads = args.cpu_threads or os.cpu_count() or 1
    times, last = [], None
    for k in range(args.warmup + args.steps):
        t_step = 0.0
        for bj in bs:
            res, total, setup = cpu.solve(rp, ci, val, bj, threads)
            t_step += total
            if bj is b:
                last = (res, total, setup)
        if k >= args.warmup:
            times.append(t_step)
    res, total, setup = last
    if setup is None:
        setup = cpu.setup_seconds(rp, ci, val, b, threads)
    true_res = float(np.linalg.norm(b - _spmv_host(rp, ci, val, res.x)) / np.linalg.norm(b))
    r1, t1, s1 = cpu.solve(rp, ci, val, b, 1)
    if s1 is None:
        s1 = cpu.setup_seconds(rp, ci, val, b, 1)
    sec = sum(times) / len(times)
    value = K / sec
    sample = ("%s: every step %d full solve(s) to %g (factorisation and all iterations) by the %s, SpMV on %d "
              "OpenMP threads, the rest serial as in the reference" %
              (label, K, TOL, "reference built from its sources" if cpu.use_ref else "oracle's C restatement",
               threads))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128" if np.iscomplexobj(val) else "f64",
            "data": "synthetic (seeded voxel generator)",
            "config": workload_config(label, n, nnz, mname, "fp64", K),
            "time_to_tolerance_s": total,
            "latency_ms": {"p50": float(np.percentile(times, 50) * 1e3), "p99": float(np.percentile(times, 99) * 1e3),
                           "steps": len(times)},
            "phases": dict(phases(res, total, setup), threads=threads, true_relative_residual=true_res),
            "one_thread": dict(phases(r1, t1, s1), solves_per_s=1.0 / t1),
            "host": host_info(),
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": cpu.kind, "sample": sample},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from sparsesolv_gb300 import _capi
    label, rp, ci, val, b = workload(args.workload)
    meth, pt, mname = method_args(args.method)
    n, nnz = len(rp) - 1, len(ci)
    dev = torch.device("cuda", local)
    cplx = np.iscomplexobj(val)
    tdt = torch.complex128 if cplx else torch.float64
    K = max(1, args.rhs)
    b1 = b  # the workload's own right-hand side (the CPU path solves it)
    b = np.ascontiguousarray(np.concatenate(extra_rhs(rp, ci, val, b, K)))
    # device-resident inputs
    val_d = torch.from_numpy(val).to(dev)
    b_d = torch.from_numpy(b).to(dev)
    x_d = torch.zeros(n * K, dtype=tdt, device=dev)
    # pinned host buffers for the end-to-end path
    val_h = torch.from_numpy(val).pin_memory()
    b_h = torch.from_numpy(b).pin_memory()
    x_h = torch.zeros(n * K, dtype=tdt).pin_memory()
    h = _capi.Handle(local)
    o = h.default_options()
    o.accel_factor = ALPHA
    o.precondition_type = pt
    o.is_save_residual_log = 1
    o.precision = _capi.PREC_MIXED if args.precision == "mixed" else _capi.PREC_FP64
    h.set_options(o)
    h.set_tuning(_capi.TUNE_SWEEP_MODE, args.sweep_mode)
    h.set_tuning(_capi.TUNE_BATCH_GROUP, args.batch_group)
    h.set_matrix(rp, ci, val)
    tuned = h.autotune() if args.autotune else None
    stream = torch.cuda.ExternalStream(h.stream(), device=dev)

    multi_iters = []

    def step_device():
        h.update_values_device(val_d.data_ptr())
        if K == 1:
            return h.solve_device(meth, b_d.data_ptr(), x_d.data_ptr(), conv=TOL, max_ite=MAXIT)
        ok_m, it_m, _ = h.solve_multi_device(meth, K, b_d.data_ptr(), x_d.data_ptr(), conv=TOL, max_ite=MAXIT)
        multi_iters[:] = it_m.tolist()
        return ok_m

    def step_host():
        h.update_values(val_h.numpy())
        xh = x_h.numpy()
        xh[:] = 0.0
        if K == 1:
            return h.solve(meth, b_h.numpy(), xh, conv=TOL, max_ite=MAXIT)
        return h.solve_multi(meth, b_h.numpy().reshape(K, n), xh.reshape(K, n), conv=TOL, max_ite=MAXIT)[0]

    for _ in range(args.warmup):
        ok = step_device()
    assert ok, "warm-up solve did not converge"
    iters = multi_iters[:] if K > 1 else h.iters()

    def barrier():
        torch.cuda.synchronize(dev)
        if ws > 1:
            torch.distributed.barrier()

    # ---- device-resident timed region (one event pair per step for the latency percentiles)
    clocks = Clocks(local)
    clocks.start()
    launches0 = h.launch_count()
    barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    t_host0 = time.perf_counter()
    for k in range(args.steps):
        ok = step_device() and ok
        ev[k + 1].record(stream)
    barrier()
    t_host = time.perf_counter() - t_host0
    ms = ev[0].elapsed_time(ev[-1])
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    launches = h.launch_count() - launches0
    clk = clocks.stop()
    # ---- per-kernel-class times from the same steps run again with event profiling
    h.set_profiling(True)
    for _ in range(args.steps):
        ok = step_device() and ok
    barrier()
    stats = h.kernel_stats()
    h.set_profiling(False)
    # ---- end-to-end through the C ABI with host buffers
    barrier()
    fe = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    clocks_e2e = Clocks(local)
    clocks_e2e.start()
    fe[0].record(stream)
    for k in range(args.steps):
        ok = step_host() and ok
        fe[k + 1].record(stream)
    barrier()
    clk_e2e = clocks_e2e.stop()
    ms_e2e = fe[0].elapsed_time(fe[-1])
    e2e_step_ms = [fe[k].elapsed_time(fe[k + 1]) for k in range(args.steps)]
    gpu_log = h.residual_log()
    xs = x_h.numpy().reshape(K, n).copy()
    bs = b.reshape(K, n)
    true_res = max(float(np.linalg.norm(bs[j] - _spmv_host(rp, ci, val, xs[j])) / np.linalg.norm(bs[j]))
                   for j in range(K))

    from sparsesolv_gb300 import replicas
    ms_max, ms_e2e_max = replicas.max_over_ranks([ms, ms_e2e])
    value = replicas.whole_job_rate(args.steps * K, ws, ms_max)
    e2e = replicas.whole_job_rate(args.steps * K, ws, ms_e2e_max)

    # roofline of the dominant kernel class
    dom = max(("forward sweep", "backward sweep", "spmv"), key=lambda k: stats[k][0])
    dms, dlaunch, dbytes = stats[dom]
    achieved = (dbytes / dlaunch) / (dms / dlaunch / 1e3) / 1e9 if dlaunch else 0.0
    peak, peak_kind = peaks()
    modes = ["automatic", "sync-free", "one-cluster", "one-cluster neighbour-synchronised", "one-cluster push"]
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("c128" if cplx else "f64") + ("+fp32-inner" if args.precision == "mixed" else ""),
        "data": "synthetic (seeded voxel generator)",
        "config": workload_config(label, n, nnz, mname, args.precision, K),
        "solver": {"iterations": iters, "true_relative_residual": true_res,
                   "parallelism": "replicas only" if ws > 1 else "single GPU",
                   "sweep_mode": modes[args.sweep_mode] if tuned is None else "autotuned: %s" % json.dumps(tuned),
                   "level_schedule": "computed once per sparsity pattern"},
        "time_to_tolerance_s": ms_max / args.steps / 1e3,
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                       "steps": len(step_ms)},
        "e2e": {"value": e2e, "unit": "solves/s",
                "step_ms": {"min": min(e2e_step_ms), "median": float(np.median(e2e_step_ms)), "max": max(e2e_step_ms)},
                "clocks": clk_e2e,
                "h2d_bytes_per_step": val.itemsize * nnz + 2 * b.itemsize * n * K,
                "d2h_bytes_per_step": b.itemsize * n * K},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"
                     if peak_kind == "measured" else "fallback 6.8 TB/s",
                     "traffic": None if K > 1 else NCU_TRAFFIC.get((args.workload, args.precision, sweep_kind(
                         tuned["mode"] if tuned else args.sweep_mode, np.iscomplexobj(val)), dom)),
                     "traffic_source": "ncu capture in profiles/ (per launch)", "algorithmic_bytes": dbytes / max(dlaunch, 1),
                     "launch_ms": dms / max(dlaunch, 1), "launches": dlaunch,
                     "fp64_pipe_frac": None if K > 1 else NCU_FP64_PIPE.get((args.workload, args.precision, sweep_kind(
                         tuned["mode"] if tuned else args.sweep_mode, np.iscomplexobj(val)), dom)),
                     "limit": "dependency levels swept one after another on one 16-SM cluster (about 1,400 at 80^3): "
                              "FP64 latency and issue on those SMs and cross-SM latency, not HBM bandwidth"},
        "kernel_ms_per_step": {k: v[0] / args.steps for k, v in stats.items()},
        "clocks": clk, "host_s": t_host,
    }
    if rank != 0:
        h.close()
        torch.distributed.destroy_process_group()
        return
    if ws == 1:
        # the measurements beside the headline: a failure in one is recorded in its place
        # (and on stderr) and never costs the line
        def aux(key, fn):
            try:
                line[key] = fn()
            except Exception as e:
                print("bench: %s failed: %r" % (key, e), file=sys.stderr, flush=True)
                line[key] = {"error": "%s: %s" % (type(e).__name__, e)}

        aux("new_pattern", lambda: new_pattern_solve(local, meth, pt, rp, ci, val, b1))
        if K == 1 and args.workload in WORKLOAD_CASE:
            aux("assembly", lambda: device_assembly(local, args.workload, rp, ci, val, b1))
        ref = None
        if not args.no_cpu_baseline:
            try:
                ref = cpu_baseline(line, rp, ci, val, b1, args.method, pt, args.cpu_threads)
            except Exception as e:
                print("bench: cpu_baseline failed: %r" % (e,), file=sys.stderr, flush=True)
                line["cpu_baseline"] = {"error": "%s: %s" % (type(e).__name__, e)}
            if ref is not None:
                aux("parity", lambda: parity_summary(rp, ci, val, b1, xs[0], iters if K == 1 else iters[0], gpu_log,
                                                     ref))
        if not args.no_mixed and K == 1 and args.method != "sgs" and args.precision == "fp64":
            aux("mixed", lambda: mixed_vs_fp64(h, o, step_device, stream, dev, x_d, args, ms_max / args.steps,
                                               rp, ci, val, b1, xs[0], ref))
        if not args.no_serving and args.workload == "cfg2" and K == 1:
            aux("serving", lambda: serving_measure(local, args.requests, args.slots, args.share, None, warm_runs=1,
                                                   sweep=False))
        if not args.no_batch and args.workload == "cfg2" and K == 1:
            aux("batch", lambda: batch_measure(local, args.batch_sizes, args.batch_persistent))
    print(json.dumps(line), flush=True)
    try:
        h.close()
    except Exception as e:
        print("bench: closing the handle failed: %r" % (e,), file=sys.stderr, flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def new_pattern_solve(device, meth, pt, rp, ci, val, b):
    """The first solve of a sparsity pattern the library has not seen, through
    the C ABI with host buffers: upload, pattern analysis (triangles, level
    schedules, sweep plans), factor and iterations, on a second handle once
    this process's CUDA modules are loaded; then the same solve again."""
    from sparsesolv_gb300 import _capi
    h2 = _capi.Handle(device)
    o2 = h2.default_options()
    o2.accel_factor = ALPHA
    o2.precondition_type = pt
    h2.set_options(o2)
    x = np.zeros_like(b)
    t0 = time.perf_counter()
    h2.set_matrix(rp, ci, val)
    ok = h2.solve(meth, np.ascontiguousarray(b), x, conv=TOL, max_ite=MAXIT)
    first = time.perf_counter() - t0
    x[:] = 0.0
    t0 = time.perf_counter()
    h2.solve(meth, np.ascontiguousarray(b), x, conv=TOL, max_ite=MAXIT)
    again = time.perf_counter() - t0
    h2.close()
    return {"first_solve_s": first, "same_pattern_again_s": again, "converged": bool(ok),
            "what": "ssg_set_matrix + ssg_solve with host buffers on a fresh handle: upload, pattern analysis, "
                    "factor, iterations; then the same solve again (pattern and factor cached)"}


def cpu_baseline(line, rp, ci, val, b, method, pt, cpu_threads):
    """A bounded sample of the CPU path (one full solve on all host cores, one
    on a single thread when the first took under 15 s); returns the all-core
    result, whose x also serves as the FP64 oracle solution for the parity and
    mixed-precision error figures."""
    cpu = CpuPath(method, pt)
    threads = cpu_threads or os.cpu_count() or 1
    res, total, setup = cpu.solve(rp, ci, val, b, threads)
    if setup is None:
        setup = cpu.setup_seconds(rp, ci, val, b, threads)
    entry = {"value": 1.0 / total, "unit": "solves/s", "cores": threads, "kind": cpu.kind,
             "sample": "one full solve to %g (factorisation %.2f s + %d iterations, %.1f ms each) on %d threads%s"
                       % (TOL, setup, res.iters, 1e3 * (total - setup) / max(res.iters, 1), threads,
                          "" if cpu.use_ref else ", the oracle's C restatement of the reference"),
             "phases": phases(res, total, setup), "host": host_info()}
    if total < 15.0 and threads > 1:
        r1, t1, s1 = cpu.solve(rp, ci, val, b, 1)
        if s1 is None:
            s1 = cpu.setup_seconds(rp, ci, val, b, 1)
        entry["one_thread"] = dict(phases(r1, t1, s1), solves_per_s=1.0 / t1)
    line["cpu_baseline"] = entry
    return res


def parity_summary(rp, ci, val, b, x, iters, gpu_log, ref):
    """The bench solve against the FP64 oracle solve of the same method, shift and
    right-hand side: iteration counts, residual-log prefix, distance of x."""
    k = min(len(gpu_log), len(ref.log), 40)
    lg = np.asarray(gpu_log[:k])
    rl = np.asarray(ref.log[:k])
    A_dx = _spmv_host(rp, ci, val, x - ref.x)
    return {"oracle": "FP64 oracle solve of the same system, method, shift and tolerance (cpu_baseline's solve)",
            "oracle_iterations": int(ref.iters), "gpu_iterations": int(iters),
            "iterations_rel_diff": abs(int(iters) - int(ref.iters)) / max(int(ref.iters), 1),
            "log_prefix_entries": int(k),
            "log_prefix_max_rel_diff": float(np.max(np.abs(lg - rl) / np.abs(rl))) if k else None,
            "x_rel_diff": float(np.linalg.norm(x - ref.x) / np.linalg.norm(ref.x)),
            "A_dx_over_b": float(np.linalg.norm(A_dx) / np.linalg.norm(b))}


def mixed_vs_fp64(h, o, step_device, stream, dev, x_d, args, fp64_ms, rp, ci, val, b, x64, ref):
    """The same solve in mixed precision (FP32 inner ICCG / IC-MRTR inside FP64
    refinement on the true residual) on the same handle and matrix."""
    import torch
    from sparsesolv_gb300 import _capi
    o.precision = _capi.PREC_MIXED
    h.set_options(o)
    try:
        for _ in range(2):
            ok = step_device()
        M = max(3, args.steps // 4)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(M):
            ok = step_device() and ok
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / M
        inner = h.iters()
        outer = len(h.residual_log()) - 1
        xm = x_d.cpu().numpy()[:len(b)].copy()
    finally:
        o.precision = _capi.PREC_FP64
        h.set_options(o)
    nb = np.linalg.norm(b)
    out = {"time_to_tolerance_s": ms / 1e3, "solves_per_s": 1e3 / ms, "steps": M, "converged": bool(ok),
           "speedup_vs_fp64": fp64_ms / ms, "inner_iterations": int(inner), "refinement_steps": int(outer),
           "true_relative_residual": float(np.linalg.norm(b - _spmv_host(rp, ci, val, xm)) / nb),
           "vs_gpu_fp64": {"x_rel_diff": float(np.linalg.norm(xm - x64) / np.linalg.norm(x64)),
                           "A_dx_over_b": float(np.linalg.norm(_spmv_host(rp, ci, val, xm - x64)) / nb)}}
    if ref is not None:
        out["vs_fp64_oracle"] = {"x_rel_diff": float(np.linalg.norm(xm - ref.x) / np.linalg.norm(ref.x)),
                                 "A_dx_over_b": float(np.linalg.norm(_spmv_host(rp, ci, val, xm - ref.x)) / nb)}
    return out


def run_batch(args):
    """256 curl-curl systems, N ~ U{8..32}, 4 coil right-hand sides each, as
    one batch (every system x right-hand side an instance in shared launches),
    ICCG with alpha 1.1 to 1e-8. A step re-factors every system and solves
    every instance; the pattern analysis of the batch is done once."""
    import torch
    from sparsesolv_gb300 import _capi, replicas, voxel
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lo, hi = (int(v) for v in args.batch_sizes.split(","))
    cases = voxel.batched_cases(lo=lo, hi=hi)
    mine = replicas.assign_systems([c.size()[1] for c, _ in cases], ws)[rank]
    systems = []
    for i in mine:
        case, coils = cases[i]
        systems.append(case.assemble(coils_list=coils))
    bt = _capi.Batch(local)
    bt.set_precision(_capi.PREC_MIXED if args.precision == "mixed" else _capi.PREC_FP64)
    bt.set_persistent(args.batch_persistent)
    for rp, ci, va, B in systems:
        bt.add(rp, ci, va, B)
    inst = sum(len(B) for _, _, _, B in systems)
    tuned = bt.autotune() if args.autotune else None
    t0 = time.perf_counter()
    bt.start(_capi.METHOD_ICCG, ALPHA, conv=TOL, max_ite=MAXIT)
    bt.wait()
    t_first = time.perf_counter() - t0
    for _ in range(max(0, args.warmup - 1)):
        bt.start(_capi.METHOD_ICCG, ALPHA, conv=TOL, max_ite=MAXIT)
        bt.wait()
    stream = torch.cuda.ExternalStream(bt.stream(), device=dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if ws > 1:
            torch.distributed.barrier()

    clocks = Clocks(local)
    clocks.start()
    launches0 = bt.lib.ssg_launch_count()
    barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    for k in range(args.steps):
        bt.start(_capi.METHOD_ICCG, ALPHA, conv=TOL, max_ite=MAXIT)
        bt.wait()
        ev[k + 1].record(stream)
    barrier()
    ms = ev[0].elapsed_time(ev[-1])
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    launches = bt.lib.ssg_launch_count() - launches0
    clk = clocks.stop()
    bt.set_profiling(True)
    bt.start(_capi.METHOD_ICCG, ALPHA, conv=TOL, max_ite=MAXIT)
    bt.wait()
    stats = bt.kernel_stats()
    bt.set_profiling(False)
    iters, conv_all = [], True
    for k in range(len(systems)):
        _, it, _, ok = bt.result(k)
        iters.extend(int(v) for v in it)
        conv_all = conv_all and ok
    # end to end: new right-hand sides from the host every step, solutions back to the host
    barrier()
    t0 = time.perf_counter()
    h2d = d2h = 0
    for _ in range(args.steps):
        for k, (_, _, _, B) in enumerate(systems):
            bt.set_rhs(k, B)
            h2d += B.nbytes
        bt.start(_capi.METHOD_ICCG, ALPHA, conv=TOL, max_ite=MAXIT)
        bt.wait()
        for k in range(len(systems)):
            X = bt.result(k)[0]
            d2h += X.nbytes
    barrier()
    ms_e2e = (time.perf_counter() - t0) * 1e3
    ms_max, ms_e2e_max = replicas.max_over_ranks([ms, ms_e2e])
    total_inst = inst * ws
    value = total_inst * args.steps / (ms_max / 1e3)
    e2e = total_inst * args.steps / (ms_e2e_max / 1e3)
    # plain FP64 GPU path: the same instances one at a time through a handle (a sample)
    h = _capi.Handle(local)
    o = h.default_options()
    o.accel_factor = ALPHA
    h.set_options(o)
    sample = list(range(0, len(systems), max(1, len(systems) // 8)))[:8]
    t_seq, n_seq = 0.0, 0
    for k in sample:
        rp, ci, va, B = systems[k]
        h.set_matrix(rp, ci, va)
        for j in range(len(B)):
            x = np.zeros_like(B[j])
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            h.solve(_capi.METHOD_ICCG, np.ascontiguousarray(B[j]), x, conv=TOL, max_ite=MAXIT)
            t_seq += time.perf_counter() - t0
            n_seq += 1
    h.close()
    seq_rate = n_seq / t_seq
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    line = {
        "metric": "batched solves/s (one solve = one system x right-hand side to 1e-8)", "value": value,
        "unit": "solves/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f64" + ("+fp32-inner" if args.precision == "mixed" else ""),
        "data": "synthetic (seeded voxel generator)",
        "config": {"workload": "256 curl-curl systems, N ~ U{%d..%d} voxels, 4 coil right-hand sides each" % (lo, hi),
                   "iterations_engine": "persistent (one CTA per instance) where every instance has at most "
                                        "16,384 rows, else launches per phase" if args.batch_persistent
                   else "launches per phase (CUDA graphs)",
                   "instances": total_inst, "rows": int(sum(len(B) * (len(rp) - 1) for rp, _, _, B in systems)),
                   "method": "shifted ICCG", "alpha": ALPHA, "tolerance": TOL, "converged": conv_all,
                   "sweep_schedule": "autotuned: %s" % json.dumps(tuned) if tuned else "fixed (8 lanes a row)",
                   "precision": args.precision,
                   "iterations": {"min": min(iters), "median": float(np.median(iters)), "max": max(iters)},
                   "factor": "recomputed every step", "pattern_analysis_s": t_first,
                   "parallelism": "replicas only" if ws > 1 else "single GPU"},
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": h2d // max(1, args.steps),
                "d2h_bytes_per_step": d2h // max(1, args.steps)},
        "gpu_launches": int(launches),
        "kernel_ms_per_step": {k: v[0] for k, v in stats.items()},
        "kernel_gbs": {k: (v[2] / (v[0] / 1e3) / 1e9 if v[0] else 0.0) for k, v in stats.items()},
        "plain_gpu_sequential": {"value": seq_rate, "unit": "solves/s", "sample_instances": n_seq,
                                 "ratio": value / seq_rate},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def batch_measure(local, sizes, persistent, steps=2):
    """The 256-system batch (the --workload cfg4 line's workload: curl-curl systems
    of N ~ U{8..32} voxels a side, 4 coil right-hand sides each, ICCG alpha 1.1 to
    1e-8) in FP64 and in mixed precision: instances solved per second over `steps`
    steps after a warm step, CUDA events on the batch's stream, each step
    re-factoring every system. The full line (latency, e2e, plain GPU ratio) is
    --workload cfg4's."""
    import torch
    from sparsesolv_gb300 import _capi, voxel
    dev = torch.device("cuda", local)
    lo, hi = (int(v) for v in sizes.split(","))
    systems = []
    for case, coils in voxel.batched_cases(lo=lo, hi=hi):
        systems.append(case.assemble(coils_list=coils))
    out = {"workload": "256 curl-curl systems, N ~ U{%d..%d} voxels, 4 coil right-hand sides each" % (lo, hi),
           "instances": int(sum(len(B) for _, _, _, B in systems)), "steps": steps,
           "what": "instances solved per second, each step re-factoring every system (CUDA events)"}
    for prec in ("fp64", "mixed"):
        bt = _capi.Batch(local)
        try:
            bt.set_precision(_capi.PREC_MIXED if prec == "mixed" else _capi.PREC_FP64)
            bt.set_persistent(persistent)
            for rp, ci, va, B in systems:
                bt.add(rp, ci, va, B)
            bt.start(_capi.METHOD_ICCG, ALPHA, conv=TOL, max_ite=MAXIT)
            bt.wait()
            stream = torch.cuda.ExternalStream(bt.stream(), device=dev)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                bt.start(_capi.METHOD_ICCG, ALPHA, conv=TOL, max_ite=MAXIT)
                bt.wait()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1)
            ok = all(bt.result(k)[3] for k in range(len(systems)))
            out[prec] = {"solves_per_s": out["instances"] * steps / (ms / 1e3), "ms_per_step": ms / steps,
                         "converged": bool(ok)}
        finally:
            bt.close()
    out["mixed_vs_fp64"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    return out


def serving_measure(local, requests, slots, share, precision, warm_runs=1, sweep=True):
    """Serving stream: requests log-uniform over 1k-500k unknowns, 70% real
    ICCG / 30% complex IC-MRTR, continuous batching to 1e-8 (mixed precision
    for real requests, FP64 for complex ones unless precision says fp64 for
    all). solves/s and p50/p99 latency with every request queued at t = 0
    (saturation); with sweep, the same requests again as Poisson arrivals at
    1/4, 1/2 and 1 x that rate. The plain FP64 GPU path solves the same
    requests one after another through a handle."""
    import torch
    import scipy.sparse as sp
    from sparsesolv_gb300 import _capi, serving
    torch.cuda.set_device(local)
    base = serving.synthetic_stream(requests, rate=0.0, seed=11)
    kinds = [r.kind for r in base]
    be = serving.GpuBackend(local, precision=None if precision != "fp64" else _capi.PREC_FP64)

    def fresh(rate, seed):
        rng = np.random.default_rng(seed)
        t, out = 0.0, []
        for r in base:
            if rate > 0:
                t += rng.exponential(1.0 / rate)
            out.append(serving.Request(r.rid, t, r.row_ptr, r.col, r.val, r.b, r.kind))
        return out

    def check(reqs):
        worst = 0.0
        for r in reqs:
            A = sp.csr_matrix((r.val, r.col, r.row_ptr))
            worst = max(worst, float(np.linalg.norm(r.b - A @ r.x) / np.linalg.norm(r.b)))
        return worst

    ns = [int(v) for v in slots.split(",")]
    srv = serving.Server(be, serving.ServerConfig(slots={serving.KIND_REAL_ICCG: ns[0],
                                                        serving.KIND_COMPLEX_MRTR: ns[1]}, share=share))
    for _ in range(max(1, warm_runs)):  # warm the slots (buffers, modules)
        srv.run(fresh(0.0, 0))
    clocks = Clocks(local)
    clocks.start()
    sat = srv.run(fresh(0.0, 0))
    clk = clocks.stop()
    st_sat = serving.latency_stats(sat)
    worst = check(sat)
    rates = []
    if sweep:
        for frac in (0.25, 0.5, 1.0):
            rate = frac * st_sat["solves_per_s"]
            reqs = srv.run(fresh(rate, 1 + int(frac * 100)))
            st = serving.latency_stats(reqs)
            st["arrival_rate"] = rate
            rates.append(st)
            worst = max(worst, check(reqs))
    srv.close()
    # plain FP64 GPU path: one request after another through a handle
    h = _capi.Handle(local)
    o = h.default_options()
    o.accel_factor = 1.1
    o.precondition_type = 0
    h.set_options(o)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_lat = []
    for r in base:
        t1 = time.perf_counter()
        h.set_matrix(r.row_ptr, r.col, r.val)
        x = np.zeros_like(r.b)
        meth = _capi.METHOD_ICCG if r.kind == serving.KIND_REAL_ICCG else _capi.METHOD_MRTR
        h.solve(meth, np.ascontiguousarray(r.b), x, conv=TOL, max_ite=MAXIT)
        plain_lat.append(time.perf_counter() - t1)
    t_plain = time.perf_counter() - t0
    h.close()
    plain_rate = len(base) / t_plain
    out = {"workload": "request stream, sizes log-uniform 1k-500k unknowns, 70% real curl-curl ICCG, "
                       "30% complex eddy-current IC-MRTR, all queued at t = 0",
           "requests": len(base), "real": kinds.count(serving.KIND_REAL_ICCG),
           "complex": kinds.count(serving.KIND_COMPLEX_MRTR), "rows": int(sum(r.n for r in base)),
           "precision": ("real ICCG mixed, complex IC-MRTR fp64" if precision != "fp64" else "fp64"),
           "slots": {k: v for k, v in srv.cfg.slots.items()}, "share": share,
           "solves_per_s": st_sat["solves_per_s"], "p50_ms": st_sat["p50_ms"], "p99_ms": st_sat["p99_ms"],
           "worst_true_relative_residual": worst,
           "plain_gpu_sequential": {"solves_per_s": plain_rate,
                                    "p50_ms": float(np.percentile(plain_lat, 50) * 1e3),
                                    "p99_ms": float(np.percentile(plain_lat, 99) * 1e3)},
           "ratio_vs_plain": st_sat["solves_per_s"] / plain_rate, "clocks": clk}
    if sweep:
        out["rate_sweep"] = rates
    return out


def run_serving(args):
    """The serving stream as its own bench line (--workload cfg5)."""
    ws, rank, local = dist_env()
    if rank != 0:
        return  # one GPU serves the stream; replicas would split it by request
    m = serving_measure(local, args.requests, args.slots, args.share, args.precision,
                        warm_runs=max(1, args.warmup - 2), sweep=True)
    line = {
        "metric": "serving solves/s at saturation, p50/p99 latency (ms) over a rate sweep",
        "value": m["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": 1, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f64/c128" + ("+fp32-inner" if args.precision != "fp64" else ""),
        "data": "synthetic (seeded voxel generator)",
        "config": {"workload": m["workload"], "requests": m["requests"], "real": m["real"],
                   "complex": m["complex"], "rows": m["rows"], "tolerance": TOL, "alpha": 1.1,
                   "precision": m["precision"], "slots": m["slots"], "share": m["share"],
                   "worst_true_relative_residual": m["worst_true_relative_residual"]},
        "latency_ms": {"p50": m["p50_ms"], "p99": m["p99_ms"]},
        "rate_sweep": m["rate_sweep"],
        "plain_gpu_sequential": dict(m["plain_gpu_sequential"], ratio=m["ratio_vs_plain"]),
        "clocks": m["clocks"],
    }
    print(json.dumps(line), flush=True)


def _spmv_host(rp, ci, val, x):
    import scipy.sparse as sp
    return sp.csr_matrix((val, ci, rp), shape=(len(rp) - 1, len(rp) - 1)) @ x


def main():
    global ALPHA
    args = parse()
    ALPHA = args.alpha
    if args.cpu_threads > 0:
        # read by the CPU path's OpenMP runtime when its library loads (after this point)
        os.environ["OMP_NUM_THREADS"] = str(args.cpu_threads)
    if args.precision is None:
        args.precision = "mixed" if args.workload == "cfg5" else "fp64"
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "cfg4":
        run_batch(args)
    elif args.workload == "cfg5":
        run_serving(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
