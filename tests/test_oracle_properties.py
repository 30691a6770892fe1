"""Size-independent properties of the oracle, and its verdicts against HiGHS
on the reference's LP formulation for sampled candidates of larger configs."""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from oracle import oracle as O
from oracle import reference_lp as R


def _set(c):
    return tuple(O.mask_to_set(c["mask_lo"], c["mask_hi"]))


@pytest.mark.parametrize("make,kmax", [(P.random_n10_m43_p4, 3), (lambda: P.mpc_mpqp(1), 3), (P.illcond_n16_m62_p8, 2)])
def test_pruning_keeps_every_feasible_set(make, kmax):
    prob = P.scale_problem(make())
    ep = O.enumerate_sets(prob, k_max=kmax, nthreads=4)
    ex = O.enumerate_sets(prob, k_max=kmax, exhaustive=True, nthreads=4)
    for f in ("feasible", "optimal", "region"):
        a = {_set(c) for c in ep.cand if c[f]}
        b = {_set(c) for c in ex.cand if c[f]}
        assert a == b, f
    assert ep.n_cand + ep.n_pruned >= ep.n_cand


def test_supersets_of_infeasible_sets_are_never_checked():
    prob = P.scale_problem(P.mpc_mpqp(2))
    e = O.enumerate_sets(prob, k_max=3)
    infeasible = [frozenset(_set(c)) for c in e.cand if not c["feasible"]]
    checked = [frozenset(_set(c)) for c in e.cand]
    for s in checked:
        assert not any(i < s for i in infeasible)


def test_warm_start_chain_equals_enumeration_records():
    prob = P.scale_problem(P.random_n10_m43_p4())
    e = O.enumerate_sets(prob, k_max=3)
    rng = np.random.default_rng(3)
    for i in rng.choice(len(e.cand), 40, replace=False):
        c = e.cand[i]
        rec, _ = O.check_set(prob, _set(c))
        for f in ("feasible", "optimal", "region", "lp1_pivots"):
            assert rec[f] == c[f], f
        assert rec["z"] == c["z"] and (rec["t"] == c["t"] or (np.isnan(rec["t"]) and np.isnan(c["t"])))


def test_budget_stops_at_the_first_level_that_does_not_fit():
    prob = P.scale_problem(P.random_n10_m43_p4())
    full = O.enumerate_sets(prob, k_max=3, keep_records=True)
    per_level = np.bincount(full.cand["level"])
    cum = np.cumsum(per_level)
    budget = int(cum[2]) + 5
    e = O.enumerate_sets(prob, k_max=3, budget=budget, keep_records=False)
    assert e.truncated == 1 and e.n_cand == cum[2]


@pytest.mark.parametrize("make,kmax,n", [(P.random_n12_m62_p6, 2, 120), (lambda: P.mpc_mpqp(4), 3, 120),
                                         (lambda: P.batch_member(9), 2, 120)])
def test_verdicts_match_highs_on_reference_formulation(make, kmax, n):
    prob = P.scale_problem(make())
    mats = R.build_lp_matrices(prob)
    e = O.enumerate_sets(prob, k_max=kmax)
    rng = np.random.default_rng(0)
    idx = np.unique(np.concatenate([rng.choice(len(e.cand), min(n, len(e.cand)), replace=False),
                                    np.nonzero(e.cand["optimal"])[0][:40], np.nonzero(e.cand["feasible"] == 0)[0][:40]]))
    for i in idx:
        c = e.cand[i]
        S = _set(c)
        z = R.lp1_value(mats, S)
        assert (z <= 1e-9) == bool(c["feasible"]), (S, z, c["z"])
        if c["feasible"] and c["licq"]:
            t = R.lp2_value(mats, S)
            assert (t > 1e-9) == bool(c["optimal"]), (S, t, c["t"])
            if np.isfinite(t):
                assert abs(t - c["t"]) <= 1e-7 * max(1.0, abs(t))
