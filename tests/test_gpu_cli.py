"""The command-line program (bin/squirmer_bem, the counterpart of the
reference's squirmer_bem, src/main.cpp:27-175) run on the reference's own
input files, its CSVs compared with the results the reference stored in its
repository (tests/golden/ref_outputs.json, copied by make_golden.py):

  inputs/duct_flow.in           -> outputs/duct_flow/{flow_rate,profile,panels}.csv
  inputs/squirmer_kinematics.in -> outputs/reference/squirmer/offaxis.csv
                                   (a/R = 0.3, level 3, n_theta = 36, six beta)
  kinematics on the axis        -> outputs/reference/squirmer/axis.csv
  inputs/squirmer_field.in      -> outputs/reference/squirmer/field.csv (with the
                                   grid of that file: |z| <= 2.2 R)

The stored files carry 10 significant digits, so values are compared to
2e-9 relative, with an absolute floor of 1e-10 of the file's largest velocity
or traction for entries that are round-off in both implementations (e.g. the
transverse velocity on the axis, ~1e-17).  Comment and header lines must be
byte-identical where the reference's program writes them."""
import io
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden

pytestmark = pytest.mark.gpu

EXE = os.path.join(ROOT, "squirmer-bem-3dtube_gb300", "bin", "squirmer_bem")


@pytest.fixture(scope="module")
def stored():
    if not os.path.exists(EXE):
        pytest.fail("bin/squirmer_bem not built (run build())")
    return golden("ref_outputs")


def run(tmp_path, stored, name, *overrides):
    inp = tmp_path / os.path.basename(name)
    inp.write_text(stored[name])
    out = tmp_path / "out"
    r = subprocess.run([EXE, str(inp), "output_dir=" + str(out), *overrides], capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr
    return out, r.stdout


def split(text):
    """comment lines, header, numeric rows of a CSV written by Csv"""
    lines = text.splitlines()
    comments = [l for l in lines if l.startswith("#")]
    body = [l for l in lines if not l.startswith("#")]
    rows = np.loadtxt(io.StringIO("\n".join(body[1:])), delimiter=",", ndmin=2) if len(body) > 1 else None
    return comments, body[0], rows


def close(got, ref, cols=None, scale=None):
    got, ref = np.asarray(got, float), np.asarray(ref, float)
    assert got.shape == ref.shape
    nan = np.isnan(ref)
    np.testing.assert_array_equal(np.isnan(got), nan)
    s = np.nanmax(np.abs(ref)) if scale is None else scale
    np.testing.assert_allclose(got[~nan], ref[~nan], rtol=2e-9, atol=1e-10 * s)


def test_duct_mode_matches_stored_outputs(tmp_path, stored):
    out, log = run(tmp_path, stored, "inputs/duct_flow.in")
    assert "1680 panels, 5040 unknowns" in log
    for name in ("flow_rate", "profile", "panels"):
        got = (out / (name + ".csv")).read_text()
        c1, h1, r1 = split(got)
        c2, h2, r2 = split(stored["outputs/duct_flow/%s.csv" % name])
        assert (c1, h1) == (c2, h2), name
        if name == "flow_rate":
            close(r1[:, :3], r2[:, :3])
            np.testing.assert_allclose(r1[:, 3], r2[:, 3], rtol=1e-6)  # |Q - Qx| / Qx: 3 digits cancel
        elif name == "profile":
            close(r1, r2, scale=np.max(np.abs(r2[:, 4:])))
        else:  # geometry columns print identically; u and f to 10 digits
            assert got.splitlines()[1].split(",")[:8] == stored["outputs/duct_flow/panels.csv"].splitlines()[1].split(",")[:8]
            close(r1[:, :8], r2[:, :8])
            close(r1[:, 8:], r2[:, 8:], scale=np.max(np.abs(r2[:, 8:])))


def test_kinematics_mode_matches_stored_offaxis(tmp_path, stored):
    out, _ = run(tmp_path, stored, "inputs/squirmer_kinematics.in")
    comments, header, rows = split((out / "kinematics.csv").read_text())
    assert header == ("a_over_R,beta,panels,UB1x,UB1y,UB1z,OB1x,OB1y,OB1z,UB2x,UB2y,UB2z,OB2x,OB2y,OB2z,"
                      "drag_K,seconds")
    assert comments[0].startswith("# U, Omega for B1=1 (neutral mode) and B2=1 (dipole mode)")
    _, h, ref = split(stored["outputs/reference/squirmer/offaxis.csv"])
    assert h == "beta,UB1x,UB1z,OB1y,UB2x,UB2z,OB2y"
    got = rows[:, [1, 3, 5, 7, 9, 11, 13]]  # beta, UB1x, UB1z, OB1y, UB2x, UB2z, OB2y
    close(got, ref, scale=0.6314)
    assert np.isfinite(rows[0, 15]) and np.all(np.isnan(rows[1:, 15]))  # towed drag on the axis only


def test_kinematics_mode_on_axis_matches_stored_axis(tmp_path, stored):
    out, _ = run(tmp_path, stored, "inputs/squirmer_kinematics.in", "n_theta=24", "beta=0",
                 "a_over_R=0.1 0.2 0.3 0.4 0.5 0.6")
    _, _, rows = split((out / "kinematics.csv").read_text())
    _, h, ref = split(stored["outputs/reference/squirmer/axis.csv"])
    assert h == "a_over_R,drag_K,drag_K_HS,U_B1,U_B2"
    close(rows[:, [0, 15, 5, 11]], ref[:, [0, 1, 3, 4]], scale=1.0)


def test_kinematics_mode_mixed_precision(tmp_path, stored):
    """the same input on the mixed-precision path: U, Omega within 1e-6 of the
    stored FP64 results (norm-wise over each row's two modes)"""
    out, _ = run(tmp_path, stored, "inputs/squirmer_kinematics.in", "precision=mixed")
    _, _, rows = split((out / "kinematics.csv").read_text())
    _, _, ref = split(stored["outputs/reference/squirmer/offaxis.csv"])
    got = rows[:, [3, 5, 7, 9, 11, 13]]
    err = np.linalg.norm(got - ref[:, 1:], axis=1) / np.linalg.norm(ref[:, 1:], axis=1)
    assert np.all(err < 1e-6), err


def test_field_mode_matches_stored_field(tmp_path, stored):
    R = 1.0 / 0.3
    out, _ = run(tmp_path, stored, "inputs/squirmer_field.in", "z_extent=%r" % (2.2 * R))
    c1, h1, b1 = split((out / "field_B1.csv").read_text())
    _, _, b2 = split((out / "field_B2.csv").read_text())
    assert h1 == "x,z,ux,uy,uz"
    assert c1[0].startswith("# lab-frame velocity in the plane y=0 for B1=1; points inside the sphere are NaN.")
    _, h, ref = split(stored["outputs/reference/squirmer/field.csv"])
    assert h == "x,z,ux_B1,uz_B1,ux_B2,uz_B2"
    got = np.column_stack([b1[:, 0], b1[:, 1], b1[:, 2], b1[:, 4], b2[:, 2], b2[:, 4]])
    close(got[:, :2], ref[:, :2])
    close(got[:, 2:], ref[:, 2:], scale=2.0 / 3)
    _, _, info = split((out / "field_info.csv").read_text())
    assert abs(info[0, 3] - 0.6313900133) < 1e-9  # U_B1 on the axis at a/R = 0.3 (axis.csv)


def test_unknown_mode_fails_cleanly(tmp_path):
    if not os.path.exists(EXE):
        pytest.fail("bin/squirmer_bem not built (run build())")
    inp = tmp_path / "bad.in"
    inp.write_text("mode = nonsense\n")
    r = subprocess.run([EXE, str(inp), "output_dir=" + str(tmp_path / "o")], capture_output=True, text=True)
    assert r.returncode == 1
    assert "unknown mode 'nonsense'" in r.stderr
