"""The drop-in C++ header API on the GPU: tests/cpp/dropin_driver.cpp is
compiled against the headers and libsqbem.so, run, and its results compared
with fixtures written by the reference."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden

pytestmark = pytest.mark.gpu

LIBDIR = os.path.join(ROOT, "squirmer-bem-3dtube_gb300", "lib")


def test_dropin_driver(tmp_path):
    exe = tmp_path / "dropin_driver"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "squirmer-bem-3dtube_gb300", "include", "bem"),
                    os.path.join(ROOT, "tests", "cpp", "dropin_driver.cpp"), "-L" + LIBDIR, "-lsqbem",
                    "-Wl,-rpath," + LIBDIR, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path)], check=True, capture_output=True, text=True, timeout=600).stdout
    r = json.loads(out)
    d = golden("duct_small")
    assert r["duct_P"] == d["P"]
    np.testing.assert_allclose(r["duct_Q"], d["Q"], rtol=1e-10)
    s = golden("swim_small")["offaxis"]
    got = np.concatenate([r["U_B1"], r["Om_B1"], r["U_B2"], r["Om_B2"]])
    ref = np.concatenate([s["B1"]["U"], s["B1"]["Om"], s["B2"]["U"], s["B2"]["Om"]])
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-10
    assert abs(r["drag_K"] - s["drag_K"]) < 1e-10 * s["drag_K"]
    assert r["list"] == [0.5, 1, 2]
    t = golden("traj")
    assert r["traj_status"] == t["status"]
    lines = [l for l in open(tmp_path / "dropin_traj.csv").read().splitlines()]
    ref_lines = [l for l in t["csv"].split("\n") if l]
    assert lines[:2] == ref_lines[:2]
    got_rows = np.array([[float(x) for x in l.split(",")] for l in lines[2:]])
    ref_rows = np.array([[float(x) for x in l.split(",")] for l in ref_lines[2:]])
    np.testing.assert_allclose(got_rows, ref_rows, rtol=2e-9, atol=1e-12)
