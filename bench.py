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


# FP64 rate of the GB300 (TFLOP/s): a DFMA / DMMA throughput probe measured
# 0.99-1.05; MEASURED_PEAKS.json carries no FP64 figure.
FP64_PEAK_TFLOPS = 1.0


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


def _cpu_init():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    orc.lib()


def _cpu_wait(seconds):
    time.sleep(seconds)
    return 0


def _cpu_worker(inst):
    """One instance through the oracle in a pool process."""
    import oracle as orc
    cpu_solve(orc, inst)
    return inst["sphere_level"]


class CpuPool:
    """The reference algorithm's throughput on all host cores: one spawned
    process per core, whole instances each, BLAS on one thread per process
    (independent solves, as the instances of a sweep are)."""

    def __init__(self):
        import multiprocessing as mp
        _cpu_init()  # builds the oracle here if needed, before the workers load it
        self.n = os.cpu_count() or 1
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

    def run(self, insts):
        t0 = time.perf_counter()
        levels = self.pool.map(_cpu_worker, insts, chunksize=1)
        return len(insts), time.perf_counter() - t0, levels

    def close(self):
        self.pool.close()
        self.pool.join()


def cpu_baseline(insts, name):
    """The reference algorithm on the host cores: throughput with one instance
    per process on every core, and the reference as shipped (one process:
    single-threaded assembly, BLAS on all threads) on a short sample."""
    pool = CpuPool()
    n, dt, levels = pool.run([insts[q % len(insts)] for q in range(pool.n)])
    pool.close()
    n1, dt1, levels1 = cpu_sample(insts, 8.0)
    return {"value": n / dt, "unit": "solves/s", "cores": pool.n, "kind": "port",
            "sample": "first %d instances of the %s workload (levels %s), one per process on %d processes; "
                      "oracle: C assembly and scipy LAPACK, one BLAS thread each" % (n, name, levels, pool.n),
            "as_shipped": {"value": n1 / dt1, "unit": "solves/s",
                           "sample": "first %d instance(s) in one process: single-threaded assembly as in the "
                                     "reference, scipy LAPACK on all threads (levels %s)" % (n1, levels1)}}


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return
    insts = workload(args.workload, args.instances)
    pool = CpuPool()
    cores = pool.n
    # each step: one instance per process (cycling through the workload)
    batch = lambda k: [insts[(k * cores + q) % len(insts)] for q in range(cores)]
    for k in range(max(args.warmup, 1)):  # untimed
        pool.run(batch(k))
    t0 = time.perf_counter()
    n = 0
    for k in range(args.steps):
        n += pool.run(batch(args.warmup + k))[0]
    dt = time.perf_counter() - t0
    pool.close()
    v = n / dt
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(args, insts, ws),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": "%d instances of the %s workload, %d per step, one per process on %d "
                                       "processes (oracle: C assembly and scipy LAPACK, one BLAS thread each)"
                                       % (n, args.workload, cores, cores)},
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
        rk_steps = 2  # RK4 steps per bench step (4 evaluations each)
        for _ in range(args.warmup):
            sqbem.trajectory_ensemble(y0, alpha, P, rk_steps, scheme=1, precision=prec)
        clocks.start()
        gpu_s, wall0, solves, states = 0.0, time.perf_counter(), 0, None
        for _ in range(args.steps):
            states, U, Om, status, secs = sqbem.trajectory_ensemble(y0, alpha, P, rk_steps, scheme=1, precision=prec)
            gpu_s += secs
            solves += 4 * rk_steps * len(w)
        wall = time.perf_counter() - wall0
        clk = clocks.stop()
        u, fsecs = sqbem.ensemble_field(states[:, -1, :], alpha, P, 25, 25, 41, 7.0, precision=prec)
        pts = int(np.sum(~np.isnan(u[..., 0])))
        line = {"metric": "trajectory-ensemble BEM solves/sec (each solve: swimmer re-assembly, Schur and the two "
                          "slip modes against the shared tube inverse)", "value": solves / gpu_s, "unit": "solves/s",
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * gpu_s / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32/bf16x3+f64" if prec == sqbem.MIXED else "f64", "data": "synthetic",
                "config": {"workload": "ensemble (%d swimmers, a/R = %.1f, level %d, n_theta = %d, RK4 dt = %g, "
                                       "%d steps per call; the tube factored once per call)"
                                       % (len(w), w[0]["a_over_R"], w[0]["sphere_level"], w[0]["n_theta"], w[0]["dt"],
                                          rk_steps)},
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
    for _ in range(args.warmup):  # >= 3 for a valid bench line
        sqbem.kinematics_batch(insts, prec)
    sqbem.kernel_stats_enable(True)
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
    # dominant kernel class of the timed region
    stats = {c: sqbem.kernel_stats(c) for c in sqbem.kernel_stats_classes()}
    sqbem.kernel_stats_enable(False)

    def roofline_of(st, note):
        top = max(st, key=lambda c: st[c][1]) if st else None
        if not top:
            return None
        nl, secs, fl, by = st[top]
        if top in ("tc_gemm",):
            achieved, peak, unit, bound = fl / secs / 1e12, peaks["bf16_tflops"], "TFLOP/s", "tensor"
        elif top == "dgemm":
            achieved, peak, unit, bound = fl / secs / 1e12, FP64_PEAK_TFLOPS, "TFLOP/s (fp64)", "tensor"
        else:
            achieved, peak, unit, bound = by / secs / 1e9, peaks["hbm_gbs"], "GB/s", "hbm"
        return {"kernel": top, "bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
                "frac": achieved / peak, "traffic": traffic_of(top, nl, fl), "launches": nl,
                "launch_seconds": secs, "peak_source": peaks["source"] if top != "dgemm" else "fp64 probe",
                "note": note}

    roofline = roofline_of(stats, "per-launch CUDA events over the timed region; with concurrent streams a "
                                  "launch's duration includes the kernels of other streams sharing the GPU")
    # the same classes from one extra, untimed step on a single stream: the
    # kernels' own rates, without co-scheduling
    roofline_1s, st1 = None, None
    if rank == 0 and args.impl == "gb300":
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
        roofline_1s = roofline_of(st1, "one untimed step on a single stream, per-launch CUDA events")
    # assembly throughput: far-kernel flops are credited at 7 x FLOPS_PER_EVAL (= 64,
    # csrc/assemble.cuh) per (target, panel) pair
    assembly = None
    kst = st1 if roofline_1s is not None else stats  # kernel durations without co-scheduling
    if "assemble_far" in kst:
        _, s_far, f_far, b_far = kst["assemble_far"]
        s_near = kst.get("assemble_near", (0, 0.0, 0.0, 0.0))[1]
        pairs = f_far / (7 * 64)
        steps_in = 1 if roofline_1s is not None else args.steps
        assembly = {"panel_pairs_per_step": pairs / steps_in, "pairs_per_s": pairs / (s_far + s_near),
                    "far_kernel_written_gbs": b_far / s_far / 1e9,
                    "far_kernel_frac_of_hbm": b_far / s_far / 1e9 / peaks["hbm_gbs"],
                    "seconds_far_near": [s_far, s_near]}
    # plain FP64 GPU path on the same workload: per-level samples, projected to
    # the workload's level mix; the mixed results are checked against it
    fp64 = None
    if rank == 0 and prec == sqbem.MIXED and not args.no_fp64 and args.workload == "sweep":
        import numpy as np
        per_level, errs = {}, []
        for lev in sorted({i["sphere_level"] for i in insts}):
            idx = [k for k, i in enumerate(insts) if i["sphere_level"] == lev][:6]
            sample = [insts[k] for k in idx]
            sqbem.kinematics_batch(sample[:1], sqbem.FP64)
            r64, s64 = sqbem.kinematics_batch(sample, sqbem.FP64)
            per_level[lev] = s64 / len(sample)
            for j, k in enumerate(idx):
                a, b = results[k][:12], r64[j][:12]
                errs.append(float(np.max(np.abs(a - b)) / np.max(np.abs(b))))
        t64 = sum(per_level[i["sphere_level"]] for i in insts)
        fp64 = {"value": len(insts) / t64, "unit": "solves/s",
                "sample": "6 instances per sphere level of the same workload, FP64 GPU path, projected to its "
                          "level mix", "seconds_per_solve_by_level": per_level,
                "mixed_over_fp64": (solves / gpu_s) / (len(insts) / t64) if ws == 1 else None,
                "max_rel_err_mixed_vs_fp64": max(errs)}
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
        "roofline_single_stream": roofline_1s,
        "assembly": assembly,
        "fp64_gpu": fp64,
        "cpu_baseline": cpu,
        "kernel_stats": {c: {"launches": v[0], "seconds": v[1], "flops": v[2], "bytes": v[3]}
                         for c, v in stats.items()},
        "kernel_stats_single_stream": None if st1 is None else
        {c: {"launches": v[0], "seconds": v[1], "flops": v[2], "bytes": v[3]} for c, v in st1.items()},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
