"""The reference's own programs (src/main.cpp, tests/test_*.cpp) compile and
link UNCHANGED against the drop-in headers and libsqbem.so -- and against
nothing else (no LAPACK symbols).  Needs the reference sources, so it is
skipped where they are absent."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

# the reference checkout, where oracle/Makefile finds one ("" otherwise)
REF = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "refdir"], capture_output=True,
                     text=True).stdout.strip()
LIBDIR = os.path.join(ROOT, "squirmer-bem-3dtube_gb300", "lib")
INC = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "squirmer-bem-3dtube_gb300", "include", "bem")]


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "src")), reason="reference sources not present")
@pytest.mark.parametrize("src", ["src/main.cpp", "tests/test_duct_flow.cpp", "tests/test_squirmer.cpp",
                                 "tests/test_trajectory.cpp"])
def test_reference_program_builds_against_dropin(tmp_path, src):
    if not os.path.exists(os.path.join(LIBDIR, "libsqbem.so")):
        pytest.skip("libsqbem.so not built")
    # copy next to nothing else, so quoted includes resolve through -I only
    local = tmp_path / os.path.basename(src)
    shutil.copy(os.path.join(REF, src), local)
    if src.startswith("tests/"):
        shutil.copy(os.path.join(REF, "tests", "test_common.hpp"), tmp_path / "test_common.hpp")
    exe = tmp_path / "prog"
    subprocess.run(["g++", "-std=c++17", "-O0", *INC, str(local), "-L" + LIBDIR, "-lsqbem",
                    "-Wl,-rpath," + LIBDIR, "-o", str(exe)], check=True, capture_output=True)
    undefined = subprocess.run(["nm", "-u", str(exe)], check=True, capture_output=True, text=True).stdout
    assert "sqbem_" in undefined
    for lapack in ("dgetrf_", "dgetrs_", "dgesv_", "dgemm_"):
        assert lapack not in undefined
