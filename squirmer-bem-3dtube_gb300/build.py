"""Build libsqbem.so (the CUDA library behind include/sqbem.h) for sm_103a.

    python squirmer-bem-3dtube_gb300/build.py [--force]

Compiles every csrc/*.cu in parallel with nvcc (one -gencode, sm_103a) and links
them into lib/libsqbem.so, then the command-line program cli/squirmer_bem.cpp
(host C++ over the drop-in headers) into bin/squirmer_bem.  Objects go to
_build/ (git-ignored); a source is recompiled only when it or a header changed.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib", "libsqbem.so")
CLI_SRC = os.path.join(PKG, "cli", "squirmer_bem.cpp")
CLI = os.path.join(PKG, "bin", "squirmer_bem")
CXX = os.environ.get("CXX", "g++")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
         "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(PKG, "include"), "-I" + CSRC]


def _headers():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    hs += glob.glob(os.path.join(PKG, "include", "bem", "**", "*.hpp"), recursive=True)
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = _headers()
    objs = [os.path.join(OBJ, os.path.basename(s)[:-3] + ".o") for s in srcs]

    def compile_one(pair):
        s, o = pair
        if not force and not _stale(o, [s] + hdrs):
            return None
        cmd = [NVCC] + ARCH + FLAGS + ["-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return "%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr)
        return None

    with ThreadPoolExecutor(max_workers=min(8, len(srcs)) or 1) as ex:
        errs = [e for e in ex.map(compile_one, zip(srcs, objs)) if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    if force or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    if force or _stale(CLI, [CLI_SRC, LIB] + hdrs):
        cmd = [CXX, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
               "-I" + os.path.join(PKG, "include", "bem"), CLI_SRC, "-L" + os.path.dirname(LIB), "-lsqbem",
               "-Wl,-rpath,$ORIGIN/../lib", "-o", CLI]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("building the command-line program failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
