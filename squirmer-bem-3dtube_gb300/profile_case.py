"""A small run through every kernel family of the library, for profiling.

    python squirmer-bem-3dtube_gb300/profile_case.py [--sweep LEVEL:COUNT ...] [--sweep-only]
                                                      [--stats-log PATH]

Default: two instances of the kinematics sweep in mixed precision (tube and
swimmer assembly, Fourier blocks of the tube, Schur LU and solves, refinement),
one adjoint instance (FP64 assembly, LU and the kernel-derivative contraction)
and a two-swimmer ensemble step with its 25 x 25 x 41 velocity field.
--sweep LEVEL:COUNT takes the first COUNT sweep instances with that sphere
level instead of the first two (repeatable: each is one batched call);
--sweep-only skips the adjoint and ensemble parts; --stats-log PATH appends
every launch's class, CUDA-event time and credited flops and bytes to PATH
(the library's kernel statistics).  Everything runs on one
stream, so the launch order is fixed and an ncu capture can name a launch by
its index:

    ncu --set full --clock-control none -k regex:<kernel> -s <skip> -c 1 \\
        python squirmer-bem-3dtube_gb300/profile_case.py

Needs a GPU; a few seconds without ncu.
"""
import argparse
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
os.environ.setdefault("SQBEM_STREAMS", "1")

import numpy as np  # noqa: E402

import sqbem  # noqa: E402
from sqbem import workloads  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sweep", action="append", default=[], metavar="LEVEL:COUNT")
    ap.add_argument("--sweep-only", action="store_true")
    ap.add_argument("--stats-log", default=None)
    args = ap.parse_args()
    if args.stats_log:
        os.environ["SQBEM_KSTATS_LOG"] = args.stats_log
        sqbem.kernel_stats_enable(True)
    sweep = workloads.sweep()
    if not args.sweep:
        sqbem.kinematics_batch(sweep[:2], sqbem.MIXED)
    for spec in args.sweep:
        lev, cnt = (int(x) for x in spec.split(":"))
        sqbem.kinematics_batch([d for d in sweep if d["sphere_level"] == lev][:cnt], sqbem.MIXED)
    if args.sweep_only:
        sqbem.kernel_stats_enable(False)
        print("profile case done: %d launches" % sqbem.launch_count())
        return
    sqbem.adjoint_batch(workloads.adjoint()[:1])
    w = workloads.ensemble()[:2]
    P = sqbem.TrajParams(a_over_R=0.3, dt=0.05, n_theta=24, sphere_level=2, L_over_R=4.0)
    R = 1.0 / P.a_over_R
    y0 = np.array([[d["beta0"] * (R - 1.0), 0.0, 0.0, *d["e"]] for d in w])
    alpha = np.array([d["alpha"] for d in w])
    states, _, _, _, _ = sqbem.trajectory_ensemble(y0, alpha, P, 1, scheme=1, precision=sqbem.MIXED)
    u, _ = sqbem.ensemble_field(states[:, -1, :], alpha, P, 25, 25, 41, 7.0, precision=sqbem.MIXED)
    sqbem.kernel_stats_enable(False)
    print("profile case done: max |u| = %.6g, %d launches" % (np.nanmax(np.abs(u)), sqbem.launch_count()))


if __name__ == "__main__":
    main()
