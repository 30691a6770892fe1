"""The oracle's mpLP path (Q = 0) against the reference's own LP2 and direct LP solves.

The reference names mpLP among its problem classes (README.md:5); its LP2
(main.py:102-128) keeps x as a variable, so with a zero Q block it decides
mpLP sets unchanged.  ``reference_lp.lp2_value`` solves that LP2, matrix for
matrix, with HiGHS.  The oracle's mpLP path (KKT factor of A_S A_S^T, a
null-space direction and the stationarity residual for |S| < n) must give
the same verdict on every LP1-feasible set.  Its regions are checked
against the problem itself: at random theta the LP min (c + H theta)^T x is
solved directly; theta must lie in some region and the region's law x(theta)
must reach the LP optimum.
"""
import numpy as np
import pytest
from scipy.optimize import linprog

from mpqpcudasolver_gb300 import problems as P
from oracle import oracle as O
from oracle import reference_lp as R

CASES = [(3, 10, 2, seed, h) for seed in (0, 1, 2) for h in (0.0, 1.0)] + [(4, 13, 3, 5, 1.0)]


def _prob(n, m, p, seed, h):
    return P.scale_problem(P.random_mplp(n, m, p, seed=seed, h_scale=h))


@pytest.mark.parametrize("case", CASES, ids=[f"n{c[0]}m{c[1]}p{c[2]}s{c[3]}h{c[4]:g}" for c in CASES])
def test_mplp_verdicts_match_reference_lp2(case):
    prob = _prob(*case)
    assert not prob.Q.any()
    e = O.enumerate_sets(prob, k_max=prob.n, exhaustive=True)
    mats = R.build_lp_matrices(prob)
    n_checked = n_short_opt = n_infeasible = 0
    for r in e.cand:
        if not r["feasible"]:
            continue
        S = O.mask_to_set(r["mask_lo"], r["mask_hi"])
        t_ref = R.lp2_value(mats, S)
        if np.isfinite(t_ref) and abs(t_ref - 1e-9) < 1e-6:
            continue        # inside the band where the two LP tolerances differ
        assert bool(r["optimal"]) == bool(t_ref > 1e-9), (S, r["t"], r["lp2_status"], t_ref)
        n_checked += 1
        n_short_opt += int(r["optimal"] and len(S) < prob.n)
        n_infeasible += int(r["lp2_status"] == O.INFEASIBLE)
        if len(S) < prob.n:
            assert r["region"] == 0, S        # no unique law x(theta)
    assert n_checked > 30
    if case[4] > 0:
        # a moving cost makes edges optimal along lower-dimensional theta sets
        assert n_short_opt > 0
    assert n_infeasible > 0


@pytest.mark.parametrize("seed,h", [(0, 0.0), (0, 1.0), (3, 1.0)])
def test_mplp_regions_cover_the_box_and_laws_are_optimal(seed, h):
    prob = _prob(4, 14, 2, seed, h)
    e = O.enumerate_sets(prob, k_max=prob.n)
    regions = {}
    for r in e.cand:
        if r["region"]:
            S = tuple(O.mask_to_set(r["mask_lo"], r["mask_hi"]))
            assert len(S) == prob.n
            rec, laws = O.check_set(prob, S, want_laws=True)
            assert rec["region"] == 1
            regions[S] = laws
    assert regions
    rng = np.random.default_rng(100 + seed)
    for _ in range(200):
        th = rng.uniform(-1.0, 1.0, prob.p)
        cost = prob.c + prob.H @ th
        lp = linprog(cost, A_ub=prob.A, b_ub=prob.b + prob.F @ th, bounds=[(None, None)] * prob.n, method="highs")
        assert lp.status == 0
        hit = [S for S, L in regions.items() if np.all(L["CR_As"] @ th <= L["CR_bs"] + 1e-9)]
        assert hit, th
        for S in hit:
            L = regions[S]
            x = L["parameter_A"] @ th + L["parameter_b"]
            assert np.all(prob.A @ x <= prob.b + prob.F @ th + 1e-9)
            assert abs(cost @ x - lp.fun) <= 1e-9 * max(1.0, abs(lp.fun))
            lam = L["lagrange_A"] @ th + L["lagrange_b"]
            assert np.all(lam >= -1e-9)
            # stationarity: c + H theta + A_S^T lambda = 0
            assert np.allclose(cost + prob.A[list(S)].T @ lam, 0.0, atol=1e-9)


def test_mplp_rejects_instances_beyond_the_id_range():
    # ids of the |S| < n LP2: (p + n + 2) + (m + ncp + 2n + 1) must stay <= 255
    prob = P.random_mplp(50, 110, 2, seed=0)   # 54 + 215 ids; the mpQP limit (166) would pass
    with pytest.raises(RuntimeError):
        O.check_set(prob, [0])
