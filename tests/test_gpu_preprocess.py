"""Device row reduction (``mpqp_reduce_constraints``) against the CPU restatement.

Both apply the same steps and thresholds (zero and duplicate rows, implicit
equalities, one LP per row for redundancy); the device solves the LPs with
its FP64 warp simplex, the restatement with HiGHS.  The statuses must be
identical on planted problems, on random instances, on the MPC instances
(whose state bounds are partly implied by the input bounds) and on the
ill-conditioned instance with near-duplicate rows.  The reduced problem must
then enumerate on the device exactly as the oracle enumerates it.
"""
import time

import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O
from oracle import preprocess as R

pytestmark = pytest.mark.gpu

CASES = {f"planted-{s}": (lambda s=s: R.planted_problem(s)[0]) for s in range(6)}
CASES.update({"n10m43p4": P.random_n10_m43_p4, "n12m62p6": P.random_n12_m62_p6,
              "illcond": P.illcond_n16_m62_p8, **{f"mpc-{s}": (lambda s=s: P.mpc_mpqp(s)) for s in range(4)}})


@pytest.mark.parametrize("case", list(CASES))
def test_device_reduction_equals_oracle(gpu_lib, case):
    prob = CASES[case]()
    t0 = time.perf_counter()
    status, red = solver.reduce_constraints(prob)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    want = R.reduce_rows(prob)
    t_cpu = time.perf_counter() - t0
    assert np.array_equal(status, want), (np.nonzero(status != want)[0], status[status != want], want[status != want])
    assert red.m == int(np.sum((want[:prob.m] == R.ROW_KEPT) | (want[:prob.m] == R.ROW_EQUALITY)))
    print(f"{case}: rows {prob.m}+{prob.ncp} -> {red.m}+{red.ncp}, counts {np.bincount(status, minlength=6).tolist()}, "
          f"device {t_dev*1e3:.1f} ms, HiGHS {t_cpu*1e3:.1f} ms")


def test_planted_statuses_on_the_device(gpu_lib):
    for seed in range(6):
        prob, expected = R.planted_problem(seed)
        status, _ = solver.reduce_constraints(prob)
        for row, want in expected.items():
            assert status[row] == want, (seed, row)


def test_reduced_mpc_problem_enumerates_like_the_oracle(gpu_lib):
    """After reduction the MPC instance loses its implied state bounds; the
    device enumeration of the reduced problem matches the oracle's."""
    prob = P.mpc_mpqp(0)
    _, red = solver.reduce_constraints(prob)
    assert red.m < prob.m
    red = P.scale_problem(red)
    ref = O.enumerate_sets(red, k_max=3, nthreads=4)
    res = solver.solve([red], precision=solver.FP64, k_max=3, cand_cap=1 << 18, arena_bytes=1 << 28)
    assert res.status == 0
    assert res.candidates == ref.n_cand
    assert res.total("feasible") == ref.n_feasible and res.total("optimal") == ref.n_optimal
    assert res.total("regions") == ref.n_region
