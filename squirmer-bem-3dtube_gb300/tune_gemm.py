"""Autotuner for the tile variant of the tensor-core GEMM (csrc/tc_gemm.cu).

    python squirmer-bem-3dtube_gb300/tune_gemm.py [--instances N] [--out PATH]

Runs the benchmark workload (the 128-instance kinematics sweep, mixed
precision) once per tile variant, each time with that variant forced for every
GEMM launch (SQBEM_TC_VARIANT), on a single stream, with every launch timed by
CUDA events (the library's kernel statistics and their per-launch log).  The
workload is deterministic, so the runs issue the same launches in the same
order; for every shape class -- the launch's largest K and N, bucketed -- the
variant with the smallest summed time wins.  The result is the table the
library reads at start-up (tuning/tc_gemm.txt beside lib/):

    # comments (GPU, workload, the per-class times behind each choice)
    kmax nmax variant        one row per class, finest first

A launch takes the first row with K <= kmax and N <= nmax.  Needs a GPU.
"""
import argparse
import collections
import json
import os
import re
import subprocess
import sys
import tempfile
import time

PKG = os.path.dirname(os.path.abspath(__file__))
K_EDGES = [128, 256, 512, 1024, 2048, 1 << 30]
N_EDGES = [256, 1024, 1 << 30]

RUN_ONE = r"""
import os, sys
sys.path.insert(0, %(pkg)r)
import sqbem
from sqbem import workloads
insts = workloads.sweep()[:%(n)d]
for _ in range(2):
    sqbem.kinematics_batch(insts, sqbem.MIXED)
sqbem.kernel_stats_enable(True)
sqbem.kinematics_batch(insts, sqbem.MIXED)
sqbem.kernel_stats_enable(False)
"""


def bucket(v, edges):
    for e in edges:
        if v <= e:
            return e
    return edges[-1]


def run_variant(variant, n):
    """[(kmax, nmax, microseconds)] of every GEMM launch of one step"""
    with tempfile.TemporaryDirectory() as tmp:
        log = os.path.join(tmp, "launches.log")
        env = dict(os.environ, SQBEM_TC_VARIANT=str(variant), SQBEM_STREAMS="1", SQBEM_KSTATS_LOG=log,
                   SQBEM_TC_TABLE=os.path.join(tmp, "none"))
        subprocess.run([sys.executable, "-c", RUN_ONE % {"pkg": PKG, "n": n}], check=True, env=env)
        out = []
        for line in open(log):
            f = line.split(None, 4)
            if len(f) < 5 or f[0] != "tc_gemm":
                continue
            m = re.search(r"N=(\d+) K=(\d+)", f[4])
            out.append((int(m.group(2)), int(m.group(1)), float(f[1])))
        return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=128)
    ap.add_argument("--out", default=os.path.join(PKG, "tuning", "tc_gemm.txt"))
    args = ap.parse_args()
    sys.path.insert(0, PKG)
    import ctypes
    import sqbem
    nv = ctypes.c_int(0)
    sqbem.lib().sqbem_gemm_variants(ctypes.byref(nv))
    runs = {v: run_variant(v, args.instances) for v in range(nv.value)}
    lengths = {len(r) for r in runs.values()}
    if len(lengths) != 1:
        raise SystemExit("variants issued different launch sequences: %s" % lengths)
    per_class = collections.defaultdict(lambda: collections.defaultdict(float))
    counts = collections.Counter()
    for v, launches in runs.items():
        for k, n, us in launches:
            c = (bucket(k, K_EDGES), bucket(n, N_EDGES))
            per_class[c][v] += us
            if v == 0:
                counts[c] += 1
    rows, notes = [], []
    for c in sorted(per_class):
        times = per_class[c]
        best = min(times, key=times.get)
        rows.append((c[0], c[1], best))
        notes.append("# K<=%d N<=%d: %d launches, ms per variant %s -> %d"
                     % (c[0], c[1], counts[c], json.dumps({v: round(t / 1e3, 3) for v, t in sorted(times.items())}),
                        best))
    total = {v: sum(t for _, _, t in r) / 1e3 for v, r in runs.items()}
    best_total = sum(min(per_class[c].values()) for c in per_class) / 1e3
    gpu = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader"], capture_output=True,
                         text=True).stdout.strip().splitlines()
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    with open(args.out, "w") as f:
        f.write("# tc_gemm tile-variant table, written by tune_gemm.py on %s (%s)\n"
                % (gpu[0] if gpu else "unknown GPU", time.strftime("%Y-%m-%d")))
        f.write("# workload: the kinematics sweep, first %d instances, mixed precision, one stream\n"
                % args.instances)
        f.write("# GEMM ms per step with one variant for every launch: %s; per-class best: %.3f\n"
                % (json.dumps({v: round(t, 3) for v, t in total.items()}), best_total))
        for line in notes:
            f.write(line + "\n")
        f.write("# kmax nmax variant\n")
        for k, n, v in rows:
            f.write("%d %d %d\n" % (k, n, v))
    print(open(args.out).read())


if __name__ == "__main__":
    main()
