"""CPU-side checks of the C ABI: the library loads, exports every entry point
include/sqbem.h declares, its host-side mesh generators are bit-identical to the
reference, and compute entry points fail loudly without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden

sqbem = pytest.importorskip("sqbem")


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "sqbem.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sqbem_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = sqbem.lib()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert set(names) <= set(sqbem.SIGNATURES), set(names) - set(sqbem.SIGNATURES)


def test_version_and_counter():
    assert b"sm_103a" in sqbem.lib().sqbem_version()
    assert sqbem.launch_count() >= 0


def test_meshes_bitwise_match_reference():
    g = golden("mesh")
    cases = {
        "swimmer_tube": lambda: sqbem.swimmer_tube_mesh(10.0 / 3, 40.0 / 3, 1.0, 12, 4),
        "swimmer_tube_24": lambda: sqbem.swimmer_tube_mesh(10.0 / 3, 40.0 / 3, 1.0, 24, 4),
        "duct": lambda: sqbem.tube_mesh(1.0, sqbem.uniform_z(0, 4, 6), 8, 3),
        "ico2": lambda: sqbem.icosphere(1.0, 2, (0.7, -0.1, 0.2)),
    }
    for k, fn in cases.items():
        m = fn()
        ref = g[k]
        np.testing.assert_array_equal(m.V.reshape(-1), ref["V"], err_msg=k)
        np.testing.assert_array_equal(m.normal.reshape(-1), ref["normal"], err_msg=k)
        np.testing.assert_array_equal(m.centroid.reshape(-1), ref["centroid"], err_msg=k)
        np.testing.assert_array_equal(m.area, ref["area"], err_msg=k)
        np.testing.assert_array_equal(m.h, ref["h"], err_msg=k)
        np.testing.assert_array_equal(m.tags, np.array(ref["tags"]).astype(int), err_msg=k)
    m = sqbem.icosphere(1.0, 1)
    m.translate((0.25, 0.5, -0.75))
    np.testing.assert_array_equal(m.V.reshape(-1), g["ico1_translated"]["V"])


def test_mesh_matches_oracle_other_sizes(oracle):
    for R, nth, nr in [(1 / 0.6, 24, 4), (1 / 0.1, 16, 3), (2.0, 30, 5)]:
        a = sqbem.swimmer_tube_mesh(R, 4 * R, 1.0, nth, nr)
        b = oracle.swimmer_tube_mesh(R, 4 * R, 1.0, nth, nr)
        np.testing.assert_array_equal(a.V, b.V)
        np.testing.assert_array_equal(a.tags, b.tags)
    for lev in range(5):
        np.testing.assert_array_equal(sqbem.icosphere(1.3, lev, (0.1, 0.2, -0.3)).V,
                                      oracle.icosphere(1.3, lev, (0.1, 0.2, -0.3)).V)


def test_bad_arguments_are_rejected():
    lib = sqbem.lib()
    P = ctypes.c_int(0)
    assert lib.sqbem_icosphere(-1.0, 2, None, 10, None, None, 0, ctypes.byref(P)) == sqbem.ERR_ARG
    assert b"icosphere" in lib.sqbem_last_error()
    assert lib.sqbem_swimmer_tube_mesh(1.0, 4.0, 1.0, 2, 4, None, None, 0, ctypes.byref(P)) == sqbem.ERR_ARG
    h = ctypes.c_void_p()
    assert lib.sqbem_tube_create(1.0, 4.0, 0.3, 24, 4, 1.0, 7, ctypes.byref(h)) == sqbem.ERR_ARG


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="a GPU is present")
def test_no_cpu_fallback_without_gpu():
    """Without a CUDA device every compute entry point fails loudly."""
    with pytest.raises(sqbem.BEMError) as e:
        sqbem.Tube(10 / 3, 40 / 3, 1.0, 8)
    assert e.value.code == sqbem.ERR_NO_DEVICE
    with pytest.raises(sqbem.BEMError):
        sqbem.panel_integrals(np.eye(3).reshape(1, 9), [[0, 0, 1.0]], 0)
