"""The one-set-per-thread first stage of the FP32 dual screen.

At levels with |S| <= 6 the first stage runs one set per thread
(k_opt_screen_lanes): a first pass stops each dual LP after a few pivots
(MPQP_SCREEN_CAP, default 3) and queues the set; a second pass reruns the
queued sets from the same start, stopping again after MPQP_SCREEN_CAP2
pivots (default 6; 0: uncapped), and a third pass runs those to the end; a
set that does not fit a rerun queue goes to the second stage (all region
rows) instead.  None of this may change a verdict: every "not optimal" is
re-verified from max(y, 0), and every other set is decided by a later stage
or in FP64.  So the feasible, optimal and region sets, and the FP64 t* and
r*, must not depend on the caps -- at caps 1 and 2 most sets are rerun twice
and the rerun queues overflow, at 1000 none is -- and must equal the oracle's.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = {
    "m62-k4": (lambda: [P.random_n12_m62_p6()], 4),
    "mpc4-k4": (lambda: [P.mpc_mpqp(s) for s in range(4)], 4),
    "small-full": (lambda: [P.random_mpqp(6, 16, 3, seed=s) for s in range(8)], 6),
}
FIELDS = ("candidates", "pruned", "feasible", "optimal", "regions", "feasible_digest", "optimal_digest",
          "region_digest")


@pytest.mark.parametrize("case", list(CASES))
def test_pivot_cap_and_rerun_keep_every_verdict(gpu_lib, case, monkeypatch):
    make, kmax = CASES[case]
    probs = [P.scale_problem(p) for p in make()]
    kw = dict(k_max=kmax, cand_cap=1 << 22, arena_bytes=1 << 30)
    runs = {}
    for cap in ("3", "1", "1000", "3/0"):
        c1, _, c2 = cap.partition("/")
        monkeypatch.setenv("MPQP_SCREEN_CAP", c1)
        monkeypatch.setenv("MPQP_SCREEN_CAP2", c2 or ("2" if c1 == "1" else "6"))
        runs[cap] = solver.solve(probs, precision=solver.MIXED, **kw)
        assert runs[cap].status == 0
    base = runs["3"]
    for cap in ("1", "1000", "3/0"):
        for f in FIELDS:
            assert np.array_equal(base.inst[f], runs[cap].inst[f]), (cap, f)
        a, b = base.opt, runs[cap].opt
        for f in ("mask_lo", "mask_hi", "inst", "region"):
            assert np.array_equal(a[f], b[f]), (cap, f)
        assert np.array_equal(a["t"], b["t"]) and np.array_equal(a["r"], b["r"])
    # and the oracle's sets
    for i, prob in enumerate(probs):
        e = O.enumerate_sets(prob, k_max=kmax, nthreads=4, keep_records=False)
        assert base.inst["optimal"][i] == e.n_optimal and base.inst["regions"][i] == e.n_region
    print(case, "first-stage LPs", base.total("lp2_first_stage_lps"), "iterations",
          base.total("lp2_first_stage_pivots"))
