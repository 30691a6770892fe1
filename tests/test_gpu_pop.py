"""The reference driver's own test problems through the drop-in path.

main.py:213-228 runs the 43 problems test_ids (main.py:219) of its data file
through mpqp() one call per problem and compares the region counts with
ppopt's.  tests/golden/pop_mpqp1_43.npz holds those problems, read from the
reference checkout by tests/golden/make_pop_fixture.py, with the C oracle's
region count of each (every active set to |S| = n), without and with the
row reduction that restates ppopt's steps (utils.py:165-190).  Here the
mirror of main.py's loop (host.calculate_mpqp_with_CUDA, one mpqp() call per
problem through the ctypes binding of main.py:25-50) must find the oracle's
counts, in mixed precision (the default) and in FP64, and the batched driver
the same.  Problem 90's reserved_memory of main.py:68-69 is exercised by
passing reserved_memory to every call.
"""
import os

import numpy as np
import pytest

from mpqpcudasolver_gb300 import host
from mpqpcudasolver_gb300 import problems as P

pytestmark = pytest.mark.gpu
FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pop_mpqp1_43.npz")


def _problems():
    d = np.load(FIXTURE)
    probs = []
    for i in d["ids"]:
        g = lambda k: d[f"p{i}/{k}"]
        probs.append(P.MPQP(g("Q"), g("c").ravel(), g("H"), g("A"), g("b").ravel(), g("F"), g("CRA"),
                            g("CRb").ravel()))
    return d, probs


@pytest.mark.parametrize("reduce", [False, True])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_reference_test_problems_region_counts(gpu_lib, reduce, precision):
    d, probs = _problems()
    rows, raw = host.calculate_mpqp_with_CUDA(probs, precision=precision, reduce=reduce, reserved_memory=2000)
    want = d["regions_reduced"] if reduce else d["regions_scaled"]
    got = rows[:, 1].astype(np.int64)
    bad = [(int(d["ids"][i]), int(got[i]), int(want[i])) for i in range(len(want)) if got[i] != want[i]]
    assert not bad, bad
    assert int(got.sum()) == int(want.sum())
    print(precision, "reduce" if reduce else "scale only", "regions", int(got.sum()), "GPU time",
          float(rows[:, 3].sum()))


def test_reference_test_problems_batched(gpu_lib):
    d, probs = _problems()
    rows, batches = host.calculate_mpqp_batched(probs, precision="mixed", reduce=True)
    assert np.array_equal(rows[:, 1].astype(np.int64), d["regions_reduced"])
