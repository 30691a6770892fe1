"""Levels that do not fit device memory whole.

The reference splits a level's LPs into n_splits chunks when they do not fit
(batched_simplex.cu:1141-1158; main.py:68-69,139-141 raise reserved_memory
and pass extra_batches for large problems).  Here the LP1 tableaus of a
level's feasible sets (the warm starts of the next level, about 98 % of the
memory per set) are kept while the arena has room; the children of a set kept
without one start LP1 from the root tableau.  The verdicts cannot depend on
which sets kept a tableau -- every FP32 verdict is certified or re-solved in
FP64 -- so a run in a deliberately small arena must give the same candidates,
feasible, optimal and region sets, and the same FP64 t* and r*, as the run
that keeps every tableau, in both precisions.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = {
    "m62-k4": (lambda: P.random_n12_m62_p6(), 4),
    "n10m43p4-k5": (lambda: P.random_n10_m43_p4(), 5),
    "mpc-k4": (lambda: P.mpc_mpqp(2), 4),
}


def _sorted(rec):
    rec = rec[rec["level"] >= 0]
    return rec[np.lexsort([rec["mask_lo"], rec["mask_hi"]])]


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("precision", [solver.FP64, solver.MIXED])
def test_small_arena_gives_the_same_sets(gpu_lib, case, precision):
    make, kmax = CASES[case]
    prob = P.scale_problem(make())
    ref = O.enumerate_sets(prob, k_max=kmax, nthreads=4)
    kw = dict(k_max=kmax, record=1, rec_cap=ref.n_cand + 16, cand_cap=ref.n_cand + 1024)
    whole = solver.solve([prob], precision=precision, arena_bytes=1 << 30, **kw)
    # room for roughly a tenth of the deepest stored level
    tab_bytes = (prob.m + prob.ncp + 1) * (prob.n + prob.p + 8) * 8
    small = solver.solve([prob], precision=precision, arena_bytes=max(1 << 20, ref.n_cand * tab_bytes // 40), **kw)
    assert whole.status == 0 and small.status == 0
    assert whole.split_levels == 0 and small.split_levels > 0
    assert small.total("lp1_cold") > 0 and small.total("nodes_without_tableau") > 0
    for f in ("candidates", "pruned", "feasible", "optimal", "regions", "feasible_digest", "optimal_digest",
              "region_digest"):
        assert np.array_equal(whole.inst[f], small.inst[f]), f
    a, b = _sorted(whole.rec), _sorted(small.rec)
    assert np.array_equal(a["mask_lo"], b["mask_lo"]) and np.array_equal(a["mask_hi"], b["mask_hi"])
    for f in ("feasible", "optimal", "region"):
        assert np.array_equal(a[f], b[f]), f
    opt = a["optimal"] == 1
    assert np.array_equal(a["t"][opt], b["t"][opt]) and np.array_equal(a["r"][opt], b["r"][opt])
    # and the oracle's sets
    o = _sorted(ref.cand)
    assert np.array_equal(b["feasible"], o["feasible"]) and np.array_equal(b["optimal"], o["optimal"])
    print(case, precision, "split levels", small.split_levels, "cold LP1 starts", small.total("lp1_cold"),
          "of", small.candidates)


def test_drop_in_reports_split_levels(gpu_lib, monkeypatch):
    """mpqp() (the reference's entry point) on a level that outgrows its arena
    returns the full result with n_splits > 1 instead of a capacity error."""
    from mpqpcudasolver_gb300 import host
    monkeypatch.setenv("MPQP_ARENA_BYTES", str(4 << 20))
    lib = host.load_mpqp_cuda()
    prog = host.MPQPProb.from_mpqp(P.random_n10_m43_p4())
    prog.process_constraints(scale_method=1)
    d = host.build_lp_data(prog)
    r = host.call_mpqp(lib, d, k_max=5)
    g = r.contents
    assert g.status == 0, solver.last_error()
    e = O.enumerate_sets(prog.to_mpqp(), k_max=5, nthreads=4, keep_records=False)
    assert g.n_splits > 1 and g.n_candidates == e.n_cand and g.n_final_lps == e.n_optimal
    assert g.n_regions == e.n_region
    lib.mpqp_free(r)
