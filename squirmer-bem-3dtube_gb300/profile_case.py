"""A small run through every kernel family of the library, for profiling.

    python squirmer-bem-3dtube_gb300/profile_case.py

Two instances of the kinematics sweep in mixed precision (tube and swimmer
assembly, tensor-core LU and solves, refinement), one adjoint instance (FP64
assembly, LU and the kernel-derivative contraction) and a two-swimmer ensemble
step with its 25 x 25 x 41 velocity field -- on one stream, so the launch order
is fixed and an ncu capture can name a launch by its index:

    ncu --set full --clock-control none -k regex:<kernel> -s <skip> -c 1 \\
        python squirmer-bem-3dtube_gb300/profile_case.py

Needs a GPU; a few seconds without ncu.
"""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
os.environ.setdefault("SQBEM_STREAMS", "1")

import numpy as np  # noqa: E402

import sqbem  # noqa: E402
from sqbem import workloads  # noqa: E402


def main():
    sqbem.kinematics_batch(workloads.sweep()[:2], sqbem.MIXED)
    sqbem.adjoint_batch(workloads.adjoint()[:1])
    w = workloads.ensemble()[:2]
    P = sqbem.TrajParams(a_over_R=0.3, dt=0.05, n_theta=24, sphere_level=2, L_over_R=4.0)
    R = 1.0 / P.a_over_R
    y0 = np.array([[d["beta0"] * (R - 1.0), 0.0, 0.0, *d["e"]] for d in w])
    alpha = np.array([d["alpha"] for d in w])
    states, _, _, _, _ = sqbem.trajectory_ensemble(y0, alpha, P, 1, scheme=1, precision=sqbem.MIXED)
    u, _ = sqbem.ensemble_field(states[:, -1, :], alpha, P, 25, 25, 41, 7.0, precision=sqbem.MIXED)
    print("profile case done: max |u| = %.6g, %d launches" % (np.nanmax(np.abs(u)), sqbem.launch_count()))


if __name__ == "__main__":
    main()
