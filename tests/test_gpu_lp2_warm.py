"""LP2 basis sharing (the reference's copy_basis_dual_1/2).

The reference starts the LP2 of a set from the final basis of a solved set
at Hamming distance one (batched_simplex.cu:525-590, scheduled at
:1518-1534) and resets to its initial basis when the copied basis is
singular (:65-83).  Here ``lp2_warm=1`` starts the first-stage dual LP of
each set S u {j} from its parent S's final basis, inverted on the device,
and falls back to the single-row start when that basis is singular or
infeasible.  The start changes only the path of the LP: every verdict of the
screen is re-verified from max(y, 0), and every final verdict is FP64.  So
the feasible, optimal and region sets, and the FP64 t* and r*, must equal
the default run's, and the counters must show the warm start in use.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver

pytestmark = pytest.mark.gpu

CASES = {
    "m62-k4": (lambda: [P.random_n12_m62_p6()], 4),
    "n10m43p4-k5": (lambda: [P.random_n10_m43_p4()], 5),
    "mpc4-k4": (lambda: [P.mpc_mpqp(s) for s in range(4)], 4),
    "n8m30p5-k5": (lambda: [P.random_mpqp(8, 30, 5, seed=3)], 5),
    "small-full": (lambda: [P.random_mpqp(6, 16, 3, seed=s) for s in range(8)], 6),
    "mplp-full": (lambda: [P.random_mplp(7, 22, 3, seed=4), P.random_mplp(6, 20, 3, seed=3)], 7),
}
FIELDS = ("candidates", "pruned", "feasible", "optimal", "regions", "feasible_digest", "optimal_digest",
          "region_digest", "lp2_first_stage_lps")


@pytest.mark.parametrize("case", list(CASES))
def test_basis_sharing_keeps_every_verdict(gpu_lib, case):
    make, kmax = CASES[case]
    probs = [P.scale_problem(p) for p in make()]
    kw = dict(k_max=kmax, cand_cap=1 << 22, arena_bytes=1 << 30)
    cold = solver.solve(probs, precision=solver.MIXED, **kw)
    warm = solver.solve(probs, precision=solver.MIXED, lp2_warm=1, **kw)
    assert cold.status == 0 and warm.status == 0
    for f in FIELDS:
        assert np.array_equal(cold.inst[f], warm.inst[f]), f
    a, b = cold.opt, warm.opt
    assert len(a) == len(b)
    for f in ("mask_lo", "mask_hi", "inst", "region"):
        assert np.array_equal(a[f], b[f]), f
    # r is NaN for the optimal mpLP sets with |S| < n (no Chebyshev ball: never a region)
    assert np.array_equal(a["t"], b["t"]) and np.array_equal(a["r"], b["r"], equal_nan=True)
    # the default run offers no basis; the shared run offers and uses some
    assert cold.total("lp2_warm_offered") == 0 and cold.total("lp2_warm_started") == 0
    lps = warm.total("lp2_first_stage_lps")
    offered, started = warm.total("lp2_warm_offered"), warm.total("lp2_warm_started")
    assert 0 < started <= offered <= lps
    print(case, "first-stage LPs", lps, "iterations cold", cold.total("lp2_first_stage_pivots"), "warm",
          warm.total("lp2_first_stage_pivots"), "offered", offered, "started", started)


def test_basis_sharing_option_is_checked(gpu_lib):
    with pytest.raises(solver.MpqpError):
        solver.solve([P.scale_problem(P.random_n4_m10_p2())], precision=solver.MIXED, k_max=1, lp2_warm=2)
