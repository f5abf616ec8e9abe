#!/usr/bin/env python
"""Benchmark: BEM kinematics solves/s on one GB300 (and N replicas under torchrun).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64]
                    [--workload sweep|kinematics] [--impl gb300|reference]

A step is one batch of the workload through sqbem_kinematics_batch (the C ABI):
  sweep       128 instances, a/R ~ U[0.1, 0.6], beta ~ U[0, 0.8 (1 - a/R)],
              level 2 or 3, n_theta = 24, L/R = 4 (seeded, synthetic geometry)
  kinematics  1 instance, a/R = 0.3, beta = 0, level 3, n_theta = 24, + towed drag
Each solve = tube assembly + LU, sphere blocks, Schur complement and the
force-/torque-free solve for the B1 and B2 modes.

value = solves / GPU time of the batches (CUDA events on the batch stream);
e2e   = solves / host wall-clock of the same public call, host parameters in,
        host results out (mesh generation and every copy included).
Per-instance working sets (dense blocks of 3N x 3N) exceed the 129 MB L2, so no
explicit L2 flush is done between steps.

--impl reference times the reference algorithm on the host cores instead: the
oracle's CPU restatement (C assembly plus LAPACK through scipy) on every core,
one process per core with single-threaded BLAS, each step one instance per
process from the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "squirmer-bem-3dtube_gb300")
sys.path.insert(0, PKG)

METRIC = "BEM solves/sec, batched mixed-precision vs plain FP64 on one GB300 at 1e-6 rel err"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="sweep", choices=["sweep", "kinematics", "ensemble", "adjoint"],
                    help="sweep (the headline) / kinematics: kinematics_batch; ensemble: 256 swimmers, RK4 "
                         "(plus the 25x25x41 field); adjoint: the 32-instance adjoint batch")
    ap.add_argument("--instances", type=int, default=0,
                    help="first N instances of the workload only (small cases for profiling)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 GPU comparison sample")
    ap.add_argument("--rk-steps", type=int, default=10,
                    help="ensemble workload: RK4 steps per bench step (the workload's full run is 200)")
    return ap.parse_args()


def dist_init(n):
    """torchrun: one process per GPU; host-side barrier / max only."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, ws, dist
    return 0, 1, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,memory.used")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9 and f[1].replace(".", "").isdigit():
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return out
        sm = sorted(float(r[1]) for r in rows)
        out["sm_mhz"] = sm[len(sm) // 2]
        out["sm_max_mhz"] = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower() in ("active", "1"):
                    reasons.add(nm)
        out["reasons"] = sorted(reasons)
        out["samples"] = len(rows)
        mem = [float(r[9]) for r in rows if len(r) > 9 and r[9].replace(".", "").isdigit()]
        out["device_mem_peak_mib"] = max(mem) if mem else None
        return out


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


def traffic_of(cls, launches, flops):
    """DRAM bytes per launch of a kernel class from the committed ncu summary:
    'cls dram_bytes_per_flop X' (measured on a smaller capture, scaled by the
    algorithmic flops per launch here) or 'cls dram_bytes_per_launch X'."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(p) or launches <= 0:
        return None
    for line in open(p):
        f = line.split()
        if line.startswith("#") or len(f) < 3 or f[0] != cls:
            continue
        if f[1] == "dram_bytes_per_flop":
            return float(f[2]) * flops / launches
        if f[1] == "dram_bytes_per_launch":
            return float(f[2])
    return None


def workload(name, n=0, rank=0):
    """the instances rank `rank` solves: independent seeded shards, rank 0 = the
    single-GPU workload (weak scaling: the per-GPU work is fixed)"""
    from sqbem import workloads
    w = workloads.sweep(shard=rank) if name == "sweep" else workloads.kinematics()
    return w[:n] if n > 0 else w


def config_of(args, insts, ws):
    """the workload description shared by both arms"""
    return {"workload": "%s (%d instances)" % (args.workload, len(insts)), "instances_per_step": len(insts),
            "precision": args.precision, "n_theta": 24, "L_over_R": 4,
            "l2": "per-instance working set > L2, no flush",
            "parallelism": "replicas" if ws > 1 else "single GPU"}


def cpu_solve(orc, inst):
    """One kinematics instance through the oracle (the reference's algorithm on the CPU)."""
    import numpy as np
    a, lam = 1.0, inst["a_over_R"]
    R = a / lam
    b = inst["beta"] * (R - a)
    tube = orc.Tube(R, inst["L_over_R"] * R, a, inst["n_theta"], inst["n_r"])
    s = orc.SwimmerSolver(tube, orc.icosphere(a, inst["sphere_level"], (b, 0, 0)), (b, 0, 0))
    e = np.array(inst["e"])
    m = s.solve_free([s.slip(e, 1, 0), s.slip(e, 0, 1)])
    if inst.get("towed") and abs(b) < 1e-12:
        s.force(s.solve_prescribed((0, 0, 1), (0, 0, 0)))
    return m


def cpu_sample(insts, budget_s=20.0):
    """Time the oracle on a bounded sample: instances in order until budget_s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.lib()
    t0 = time.perf_counter()
    done = 0
    levels = []
    for inst in insts:
        cpu_solve(orc, inst)
        done += 1
        levels.append(inst["sphere_level"])
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return done, dt, levels


BLAS_THREAD_VARS = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")


def host_cores():
    """CPUs this process may run on (affinity mask / cpuset), else all CPUs."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def _cpu_init():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.lib()


def _cpu_wait(seconds):
    time.sleep(seconds)
    return 0


def _cpu_worker(job):
    """One instance through the oracle in a pool process: (index, level, seconds)."""
    import oracle as orc
    k, inst = job
    t0 = time.perf_counter()
    cpu_solve(orc, inst)
    return k, inst["sphere_level"], time.perf_counter() - t0


def mix_rate(per_level, insts, cores):
    """Throughput of `cores` busy processes on the workload's level mix, from
    the mean seconds per solve at each level."""
    mean = {lev: sum(v) / len(v) for lev, v in per_level.items() if v}
    lv = [i["sphere_level"] for i in insts if i["sphere_level"] in mean]
    if not lv:
        return None
    return cores / (sum(mean[x] for x in lv) / len(lv))


class CpuPool:
    """The reference algorithm's throughput on all host cores: one spawned
    process per core, whole instances each, BLAS on one thread per process
    (independent solves, as the instances of a sweep are).  Instances stream
    through the pool with no barrier between them, so every core stays busy."""

    def __init__(self):
        import multiprocessing as mp
        _cpu_init()  # builds the oracle here if needed, before the workers load it
        self.n = host_cores()
        saved = {k: os.environ.get(k) for k in BLAS_THREAD_VARS}
        for k in BLAS_THREAD_VARS:
            os.environ[k] = "1"  # read by the children's BLAS at load time
        try:
            self.pool = mp.get_context("spawn").Pool(self.n, initializer=_cpu_init)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        self.pool.map(_cpu_wait, [0.5] * self.n, chunksize=1)  # every worker up and loaded

    def stream(self, insts):
        """Solve insts (in order, all cores busy); returns [(index, level,
        seconds)] in completion order and the wall time."""
        t0 = time.perf_counter()
        out = list(self.pool.imap_unordered(_cpu_worker, list(enumerate(insts)), chunksize=1))
        return out, time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()


def cpu_baseline(insts, name):
    """The reference algorithm on the host cores: throughput with every core
    busy (two instances per core, streamed; each solve timed, projected to the
    workload's level mix), and the reference as shipped (one process:
    single-threaded assembly, BLAS on all threads) on a short sample."""
    pool = CpuPool()
    sample = [insts[q % len(insts)] for q in range(2 * pool.n)]
    done, wall = pool.stream(sample)
    pool.close()
    per_level = {}
    for _, lev, sec in done:
        per_level.setdefault(lev, []).append(sec)
    n1, dt1, levels1 = cpu_sample(insts, 8.0)
    return {"value": mix_rate(per_level, insts, pool.n), "unit": "solves/s", "cores": pool.n, "kind": "port",
            "sample": "first %d instances of the %s workload streamed through %d processes (all busy; oracle: C "
                      "assembly and scipy LAPACK, one BLAS thread each); each solve timed, the mean seconds per "
                      "sphere level projected to the workload's level mix" % (len(sample), name, pool.n),
            "seconds_per_solve_by_level": {lev: sum(v) / len(v) for lev, v in per_level.items()},
            "completed_over_wall": len(done) / wall,
            "as_shipped": {"value": n1 / dt1, "unit": "solves/s",
                           "sample": "first %d instance(s) in one process: single-threaded assembly as in the "
                                     "reference, scipy LAPACK on all threads (levels %s)" % (n1, levels1)}}


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return
    insts = workload(args.workload, args.instances)
    pool = CpuPool()
    cores = pool.n
    # a step is `cores` instances of the workload (in order, cycling); all steps
    # stream through the pool without a barrier between them, the warm-up
    # steps' solves first, and each solve is timed in its worker
    nw = max(args.warmup, 1) * cores
    seq = [insts[q % len(insts)] for q in range(nw + args.steps * cores)]
    done, wall = pool.stream(seq)
    pool.close()
    per_level = {}
    timed = [(k, lev, sec) for k, lev, sec in done if k >= nw]
    for _, lev, sec in timed:
        per_level.setdefault(lev, []).append(sec)
    v = mix_rate(per_level, insts, cores)
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * cores / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(args, insts, ws),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": "%d instances of the %s workload (%d per step) streamed through %d processes "
                                       "with no barrier between them (oracle: C assembly and scipy LAPACK, one BLAS "
                                       "thread each); each solve timed in its worker, the mean seconds per sphere "
                                       "level projected to the workload's level mix"
                                       % (len(timed), args.workload, cores, cores),
                             "seconds_per_solve_by_level": {lev: sum(x) / len(x) for lev, x in per_level.items()},
                             "completed_over_wall": len(done) / wall},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_aux(args, rank, ws):
    """Secondary workloads (configs 4 and 5), one JSON line each; not the headline."""
    import math
    import numpy as np
    import sqbem
    from sqbem import workloads
    prec = sqbem.MIXED if args.precision == "mixed" else sqbem.FP64
    clocks = Clocks()
    if args.workload == "ensemble":
        w = workloads.ensemble()
        if args.instances:
            w = w[:args.instances]
        R = 1.0 / w[0]["a_over_R"]
        y0 = np.array([[d["beta0"] * (R - 1.0), 0.0, 0.0, *d["e"]] for d in w])
        alpha = np.array([d["alpha"] for d in w])
        P = sqbem.TrajParams(a_over_R=w[0]["a_over_R"], dt=w[0]["dt"], n_theta=w[0]["n_theta"],
                             sphere_level=w[0]["sphere_level"], L_over_R=w[0]["L_over_R"])
        rk_steps = args.rk_steps  # RK4 steps per bench step (4 evaluations each)
        for _ in range(args.warmup):
            sqbem.trajectory_ensemble(y0, alpha, P, 1, scheme=1, precision=prec)
        builds0 = sqbem.tube_cache_stats()[0]
        clocks.start()
        gpu_s, wall0, solves, states = 0.0, time.perf_counter(), 0, None
        for _ in range(args.steps):
            sqbem.tube_cache_clear()  # every timed call assembles and factors its tube itself
            states, U, Om, status, secs = sqbem.trajectory_ensemble(y0, alpha, P, rk_steps, scheme=1, precision=prec)
            gpu_s += secs
            solves += 4 * rk_steps * len(w)
        wall = time.perf_counter() - wall0
        clk = clocks.stop()
        tube_builds = sqbem.tube_cache_stats()[0] - builds0
        u, fsecs = sqbem.ensemble_field(states[:, -1, :], alpha, P, 25, 25, 41, 7.0, precision=prec)
        pts = int(np.sum(~np.isnan(u[..., 0])))
        line = {"metric": "trajectory-ensemble BEM solves/sec (each solve: swimmer re-assembly, Schur and the two "
                          "slip modes against the shared tube's Fourier blocks)", "value": solves / gpu_s, "unit": "solves/s",
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * gpu_s / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32/bf16x3+f64" if prec == sqbem.MIXED else "f64", "data": "synthetic",
                "config": {"workload": "ensemble (%d swimmers, a/R = %.1f, level %d, n_theta = %d, RK4 dt = %g, "
                                       "%d steps per call; each timed call assembles the tube and inverts its Fourier blocks "
                                       "once (%d tube builds in the timed region), the sphere-sphere blocks once)"
                                       % (len(w), w[0]["a_over_R"], w[0]["sphere_level"], w[0]["n_theta"], w[0]["dt"],
                                          rk_steps, tube_builds)},
                "e2e": {"value": solves / wall, "unit": "solves/s"},
                "field": {"grid": [25, 25, 41], "points_evaluated": pts, "seconds": fsecs,
                          "points_per_s": pts / fsecs,
                          "note": "the field call re-solves every swimmer at its final state, then evaluates"},
                "clocks": clk}
    else:  # adjoint
        insts = workloads.adjoint()
        for _ in range(args.warmup):
            sqbem.adjoint_batch(insts[:4])
        clocks.start()
        gpu_s, wall0 = 0.0, time.perf_counter()
        for _ in range(args.steps):
            res, secs = sqbem.adjoint_batch(insts)
            gpu_s += secs
        wall = time.perf_counter() - wall0
        clk = clocks.stop()
        n = len(insts) * args.steps
        line = {"metric": "adjoint evaluations/sec (U, Omega and d(U, Omega)/dc for both slip modes, FP64)",
                "value": n / gpu_s, "unit": "instances/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * gpu_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "adjoint (32 instances, level 2, n_theta = 24)"},
                "e2e": {"value": n / wall, "unit": "instances/s"}, "clocks": clk}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, ws, dist = dist_init(args.gpus)
    if args.workload in ("ensemble", "adjoint"):
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the sweep and "
                                  "kinematics workloads only"}), flush=True)
            return
        run_aux(args, rank, ws)
        return
    if args.impl == "reference":
        run_reference(args, rank, ws, dist)
        return
    import sqbem
    prec = sqbem.MIXED if args.precision == "mixed" else sqbem.FP64
    insts = workload(args.workload, args.instances, rank)
    peaks = load_peaks()
    sqbem.set_limits(-1, -1)
    for _ in range(args.warmup):  # >= 3 for a valid bench line
        sqbem.kinematics_batch(insts, prec)
    launches0 = sqbem.launch_count()
    h2d0, d2h0 = sqbem.transfer_bytes()
    clocks = Clocks()
    barrier(dist)
    clocks.start()
    gpu_s = 0.0
    wall0 = time.perf_counter()
    results = None
    for _ in range(args.steps):
        results, secs = sqbem.kinematics_batch(insts, prec)
        gpu_s += secs
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    barrier(dist)
    launches = sqbem.launch_count() - launches0
    h2d, d2h = sqbem.transfer_bytes()
    gpu_s = allmax(dist, gpu_s)
    wall = allmax(dist, wall)
    solves = allsum(dist, float(len(insts) * args.steps))
    step_s = gpu_s / args.steps
    # the kernels' own rates: the same workload once more, untimed, on a single
    # stream, every launch bracketed by CUDA events on its stream
    st1, fp64_peak, fp32_peak = None, None, None
    if rank == 0:
        fp64_peak, fp32_peak = sqbem.pipe_rates()
        prev = os.environ.get("SQBEM_STREAMS")
        os.environ["SQBEM_STREAMS"] = "1"
        sqbem.kernel_stats_enable(True)
        sqbem.kinematics_batch(insts, prec)
        st1 = {c: sqbem.kernel_stats(c) for c in sqbem.kernel_stats_classes()}
        sqbem.kernel_stats_enable(False)
        if prev is None:
            del os.environ["SQBEM_STREAMS"]
        else:
            os.environ["SQBEM_STREAMS"] = prev

    def roofline_of(st):
        top = max(st, key=lambda c: st[c][1]) if st else None
        if not top:
            return None
        nl, secs, fl, by = st[top]
        if top == "tc_gemm":
            achieved, peak, unit, bound, src = fl / secs / 1e12, peaks["bf16_tflops"], "TFLOP/s", "tensor", \
                peaks["source"]
        elif top in ("dgemm", "assemble_near"):
            achieved, peak, unit, bound, src = fl / secs / 1e12, fp64_peak, "TFLOP/s (fp64)", "fp64", \
                "measured now (sqbem_pipe_rates)"
        else:
            achieved, peak, unit, bound, src = by / secs / 1e9, peaks["hbm_gbs"], "GB/s", "hbm", peaks["source"]
        # one step's worth of this class cannot take longer than the step
        assert secs <= step_s * 1.0001 or args.workload != "sweep" or ws > 1, \
            "%s: %.3f s of kernel time in one single-stream step > %.3f s per step" % (top, secs, step_s)
        return {"kernel": top, "bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
                "frac": achieved / peak, "traffic": traffic_of(top, nl, fl), "launches": nl,
                "launch_seconds": secs, "share_of_step": secs / step_s, "peak_source": src,
                "note": "one untimed step of the same workload on a single stream right after the timed region; "
                        "per-launch CUDA events on the launching stream; achieved = credited work / summed "
                        "launch durations"}

    roofline = roofline_of(st1) if st1 else None
    # assembly throughput: far-kernel flops are credited at 7 x FLOPS_PER_EVAL (= 64,
    # csrc/assemble.cuh) per (target, panel) pair; near-kernel flops per rule
    # from the pair counts (FP64 work: 448-point rule and self integral in mixed mode)
    assembly = None
    if st1 and "assemble_far" in st1:
        _, s_far, f_far, b_far = st1["assemble_far"]
        _, s_near, f_near, _ = st1.get("assemble_near", (0, 0.0, 0.0, 0.0))
        pairs = f_far / (7 * 64)
        mixed = prec == sqbem.MIXED
        assembly = {"panel_pairs_per_step": pairs, "pairs_per_s": pairs / (s_far + s_near),
                    "far_kernel_written_gbs": b_far / s_far / 1e9,
                    "far_kernel_frac_of_hbm": b_far / s_far / 1e9 / peaks["hbm_gbs"],
                    "far_kernel_tflops": f_far / s_far / 1e12,
                    "far_kernel_frac_of_pipe": f_far / s_far / 1e12 / (fp32_peak if mixed else fp64_peak),
                    "far_pipe": "fp32" if mixed else "fp64",
                    "near_kernel_fp64_tflops": f_near / s_near / 1e12 if s_near else None,
                    "near_kernel_frac_of_fp64": f_near / s_near / 1e12 / fp64_peak if s_near else None,
                    "seconds_far_near": [s_far, s_near],
                    "pipe_peaks_tflops": {"fp64": fp64_peak, "fp32": fp32_peak,
                                          "source": "measured now (sqbem_pipe_rates: FMA chains on every SM)"}}
    # plain FP64 GPU path on the whole workload: its rate, and every mixed
    # result compared with it (U, Omega per slip mode; sphere and wall tractions)
    fp64 = None
    if rank == 0 and prec == sqbem.MIXED and not args.no_fp64 and args.workload == "sweep":
        import numpy as np
        rm, _, fsm, ftm = sqbem.kinematics_batch(insts, sqbem.MIXED, tractions=True)
        sqbem.kinematics_batch(insts[:1], sqbem.FP64)
        r64, s64, fs64, ft64 = sqbem.kinematics_batch(insts, sqbem.FP64, tractions=True)
        # each instance is a squirmer with B2/B1 = alpha (the workload's draw):
        # U = U_B1 + alpha U_B2 and likewise Omega and the tractions
        errs = {"U": [], "Omega": [], "U_Omega_both_modes": [], "f_sphere": [], "f_tube": []}
        for k, inst in enumerate(insts):
            al = inst.get("alpha", 0.0)
            comb = lambda r, j: r[k][j:j + 3] + al * r[k][6 + j:9 + j]
            U, U64, W, W64 = comb(rm, 0), comb(r64, 0), comb(rm, 3), comb(r64, 3)
            errs["U"].append(float(np.linalg.norm(U - U64) / np.linalg.norm(U64)))
            # rotation rates in units of U/a (a = 1): Omega -> 0 on the axis
            errs["Omega"].append(float(np.linalg.norm(W - W64) / max(np.linalg.norm(W64), np.linalg.norm(U64))))
            errs["U_Omega_both_modes"].append(float(np.linalg.norm(rm[k][:12] - r64[k][:12]) /
                                                    np.linalg.norm(r64[k][:12])))
            for q, A, B in (("f_sphere", fsm[k], fs64[k]), ("f_tube", ftm[k], ft64[k])):
                if B.size:
                    fa, fb = A[0] + al * A[1], B[0] + al * B[1]
                    errs[q].append(float(np.max(np.abs(fa - fb)) / np.max(np.abs(fb))))
        per_q = {q: {"max": max(v), "median": float(np.median(v)), "count": len(v)} for q, v in errs.items() if v}
        fp64 = {"value": len(insts) / s64, "unit": "solves/s",
                "sample": "the whole workload through the FP64 GPU path (same batching)",
                "mixed_over_fp64": (solves / gpu_s) / (len(insts) / s64) if ws == 1 else None,
                "instances_compared": len(insts),
                "max_rel_err_mixed_vs_fp64": max(per_q["U"]["max"], per_q["Omega"]["max"]),
                "rel_err_mixed_vs_fp64": per_q,
                "error_norms": "per instance, for its squirmer B2/B1 = alpha: U |dU|/|U|; Omega "
                               "|dOmega|/max(|Omega|, |U|/a); U_Omega_both_modes |d(U,Omega)_B1,B2|/|(U,Omega)_B1,B2|; "
                               "f_sphere, f_tube max|df|/max|f| of f_B1 + alpha f_B2"}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(insts, args.workload)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": solves / gpu_s, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * gpu_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32/bf16x3+f64" if prec == sqbem.MIXED else "f64", "data": "synthetic",
        "config": config_of(args, insts, ws),
        "e2e": {"value": solves / wall, "unit": "solves/s", "h2d_bytes_per_step": (h2d - h2d0) / args.steps,
                "d2h_bytes_per_step": (d2h - d2h0) / args.steps},
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": roofline,
        "assembly": assembly,
        "fp64_gpu": fp64,
        "cpu_baseline": cpu,
        "kernel_stats_single_stream": None if st1 is None else
        {c: {"launches": v[0], "seconds": v[1], "flops": v[2], "bytes": v[3]} for c, v in st1.items()},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
