"""Regenerate the golden fixtures in this folder from the reference itself.

Runs ``oracle/_ref/ref_dump`` -- a dumper built by ``make -C oracle ref`` from the
UNMODIFIED reference headers (squirmer-bem-3dtube ``src/*.hpp``) linked against
scipy's bundled OpenBLAS -- once per case and stores its JSON output here.  The
reference sources are needed only to rebuild the dumper; the fixtures themselves
are committed, so the tests never touch the reference.

    make -C oracle ref && python tests/golden/make_golden.py [case ...]

Cases (all FP64, 17 significant digits):
  mesh        tube / duct / icosphere geometry (V, normal, centroid, area, h, tags)
  panel       panel_integrals (SL, DL) for self, all four rules, off-plane targets
  swim_small  small tube + sphere kinematics, towed solves, field samples,
              and the unbounded sphere
  duct_small  DuctFlow(1, 4, 8, 8, 3): Q per dP, panel u/f, interior velocity
  duct_c1     DuctFlow(1, 4, 24, 24, 6): the full duct-flow configuration
  c2          a/R = 0.3, beta = 0, level 3, n_theta = 24 (full kinematics size)
  c2_l2       level-2 cases at n_theta = 24 (on axis, off axis, tilted)
  traj        a 6-step trajectory (3 RK4 + 3 AB4) on a small mesh (CSV, 10 digits)
  ref_outputs the reference's own stored results, copied as text: the input files
              inputs/{duct_flow,squirmer_kinematics,squirmer_field}.in and the
              CSVs outputs/duct_flow/{flow_rate,profile,panels}.csv and
              outputs/reference/squirmer/{axis,offaxis,field,blake,reciprocal}.csv
              (10 digits; written by the reference's own programs)
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
DUMPER = os.path.join(HERE, "..", "..", "oracle", "_ref", "ref_dump")
CASES = ["mesh", "panel", "swim_small", "duct_small", "duct_c1", "c2", "c2_l2", "traj", "ref_outputs"]
STORED = ["inputs/duct_flow.in", "inputs/squirmer_kinematics.in", "inputs/squirmer_field.in",
          "outputs/duct_flow/flow_rate.csv", "outputs/duct_flow/profile.csv", "outputs/duct_flow/panels.csv",
          "outputs/reference/squirmer/axis.csv", "outputs/reference/squirmer/offaxis.csv",
          "outputs/reference/squirmer/field.csv", "outputs/reference/squirmer/blake.csv",
          "outputs/reference/squirmer/reciprocal.csv"]


def reference_dir():
    """the reference checkout that oracle/Makefile names"""
    ref = subprocess.run(["make", "-s", "-C", os.path.join(HERE, "..", "..", "oracle"), "refdir"],
                         capture_output=True, text=True).stdout.strip()
    if not ref:
        raise SystemExit("reference checkout not found (see oracle/Makefile)")
    return ref


def stored_outputs():
    ref = reference_dir()
    obj = {}
    for rel in STORED:
        with open(os.path.join(ref, rel)) as f:
            obj[rel] = f.read()
    return obj


def run(case):
    if case == "ref_outputs":
        obj = stored_outputs()
        with open(os.path.join(HERE, case + ".json"), "w") as f:
            json.dump(obj, f, indent=0)
        return obj
    with tempfile.TemporaryDirectory() as tmp:
        out = subprocess.run([DUMPER, case, tmp], check=True, capture_output=True, text=True,
                             env=dict(os.environ, OPENBLAS_NUM_THREADS="8"))
    obj = json.loads(out.stdout)
    with open(os.path.join(HERE, case + ".json"), "w") as f:
        json.dump(obj, f, separators=(",", ":"))
    return obj


if __name__ == "__main__":
    for c in sys.argv[1:] or CASES:
        run(c)
        print("wrote", c)
