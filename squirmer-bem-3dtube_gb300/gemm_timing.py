"""Device time of the tensor-core GEMM per tile variant on given shapes.

    python squirmer-bem-3dtube_gb300/gemm_timing.py [M,N,K,count ...]

Each shape is one grouped launch of `count` problems M x N x K with
device-resident pseudo-random split-BF16 operands (sqbem_gemm_timing: one
warm-up, then 20 launches timed with CUDA events), once with beta = 0 and once
with beta = 1 (C read and updated).  Rates are MMA flops (3 BF16 products per
element product).  Without arguments: the launch shapes of the kinematics sweep
(TRSM leaves and updates, Schur products) and three large squares.  Needs a GPU.
"""
import ctypes
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import sqbem  # noqa: E402

DEFAULT = [(128, 128, 128, 11), (128, 128, 128, 48), (128, 966, 128, 20), (128, 3846, 128, 21),
           (3840, 128, 128, 21), (128, 3846, 256, 21), (256, 3846, 256, 21), (1920, 1920, 1792, 8),
           (3840, 3840, 3968, 4), (4096, 4096, 4096, 2)]


def main():
    shapes = [tuple(int(x) for x in a.split(",")) for a in sys.argv[1:]] or DEFAULT
    lib = sqbem.lib()
    nv = ctypes.c_int(0)
    lib.sqbem_gemm_variants(ctypes.byref(nv))
    print("variant  M      N      K      count  beta   us/launch  TF/s (MMA)")
    for v in range(nv.value):
        for M, N, K, c in shapes:
            for beta in (0.0, 1.0):
                t = ctypes.c_double(0)
                if lib.sqbem_gemm_timing(v, 3, M, N, K, c, ctypes.c_float(beta), 20, ctypes.byref(t)) != 0:
                    print("v%d %s: %s" % (v, (M, N, K, c), lib.sqbem_last_error().decode()))
                    continue
                fl = 3 * 2.0 * M * N * K * c
                print("%-8d %-6d %-6d %-6d %-6d %-6g %9.2f  %8.1f" % (v, M, N, K, c, beta, t.value * 1e6,
                                                                     fl / t.value / 1e12), flush=True)


if __name__ == "__main__":
    main()
