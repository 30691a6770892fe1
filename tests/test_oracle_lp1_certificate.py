"""LP1 infeasibility has a dual certificate in the final basis.

LP1 of a set T is  min c.w  s.t.  G u + w = beta, w >= 0, u free, with c = 1
on T; every y with G^T y = 0 and y <= c bounds z*(T) >= beta.y.  The oracle
builds y from the final basis of a set's warm-start chain (y_i = c_i on the
basic slacks, the nonbasic slacks' duals from the free-variable equations).
On these instances every LP1-infeasible candidate is certified, with beta.y
equal to its z* to 1e-10 relative, and no feasible candidate is: the check a
certificate built on the device from FP32 bases is to be held to.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from oracle import oracle as O

CASES = {
    "n4m10p2-exhaustive": (lambda: P.random_n4_m10_p2(), 4, True),
    "n10m43p4-k3": (lambda: P.random_n10_m43_p4(), 3, False),
    "illcond-k4": (lambda: P.illcond_n16_m62_p8(), 4, False),   # 12 infeasible of 557,845
    "n5m14p2-k5": (lambda: P.random_mpqp(5, 14, 2, seed=13), 5, False),
}


@pytest.mark.parametrize("case", list(CASES))
def test_every_lp1_infeasible_candidate_is_certified(case):
    make, kmax, exh = CASES[case]
    prob = P.scale_problem(make())
    e = O.enumerate_sets(prob, k_max=kmax, exhaustive=exh, nthreads=8)
    cand = e.cand[e.cand["level"] >= 1]
    infeasible = cand[(cand["feasible"] == 0) & (cand["lp1_status"] == O.OPTIMAL)]
    assert len(infeasible) > 0
    tol_feas = O.default_tol().tol_feas
    for c in infeasible:
        S = O.mask_to_set(c["mask_lo"], c["mask_hi"])
        ok, bound, z, used = O.lp1_dual_bound(prob, S)
        assert ok and bound > tol_feas, (S, bound, z)
        assert abs(bound - z) <= 1e-10 * max(1.0, abs(z)), (S, bound, z)
        assert used <= len(S)
    feasible = cand[cand["feasible"] == 1]
    rng = np.random.default_rng(0)
    for c in feasible[rng.permutation(len(feasible))[:1500]]:
        S = O.mask_to_set(c["mask_lo"], c["mask_hi"])
        ok, bound, z, used = O.lp1_dual_bound(prob, S)
        assert not (ok and bound > tol_feas), (S, bound, z)
