"""Two batched calls from two host threads at the same time.

Each batched call runs its chunks on worker slots (a stream and a cache of
idle device blocks per worker index, kept across calls).  A second call that
finds a slot in use gets a stream of its own and no cache for that worker.
Both calls must give exactly what the same calls give one after the other."""
import threading

import numpy as np
import pytest

sqbem = pytest.importorskip("sqbem")
from sqbem import workloads  # noqa: E402

pytestmark = pytest.mark.gpu


def test_concurrent_batched_calls_match_sequential():
    sweep = workloads.sweep()
    a = [d for d in sweep if d["sphere_level"] == 2][:6]
    b = [d for d in sweep if d["sphere_level"] == 2][6:12]
    ref_a, _ = sqbem.kinematics_batch(a, sqbem.MIXED)
    ref_b, _ = sqbem.kinematics_batch(b, sqbem.MIXED)
    out = {}
    errors = []

    def run(key, insts):
        try:
            out[key] = sqbem.kinematics_batch(insts, sqbem.MIXED)[0]
        except Exception as e:  # reported below, in the test's thread
            errors.append(e)

    for _ in range(2):
        threads = [threading.Thread(target=run, args=("a", a)), threading.Thread(target=run, args=("b", b))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert not errors, errors
        np.testing.assert_array_equal(out["a"], ref_a)
        np.testing.assert_array_equal(out["b"], ref_b)


def test_trim_pool_between_calls():
    insts = [d for d in workloads.sweep() if d["sphere_level"] == 2][:4]
    r1, _ = sqbem.kinematics_batch(insts, sqbem.MIXED)
    sqbem.trim_pool()
    r2, _ = sqbem.kinematics_batch(insts, sqbem.MIXED)
    np.testing.assert_array_equal(r1, r2)
