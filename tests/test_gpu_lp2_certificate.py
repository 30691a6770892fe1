"""FP64 check of the FP32 dual screen's "not optimal" below its margin.

The FP32 dual screen accepts "not optimal" only when its verified bound is
below an error margin that grows with the KKT factor's conditioning.  A set
whose FP32 bound is negative but inside that margin goes to the FP64 kernel
with the screen's final dual basis; there the basis is solved again on the
FP64 rows (``lp2_cert64``) and the weak-duality bound from max(y, 0) decides
the set without the FP64 LP2 when it is clearly below zero.  The reference
decides LP2 in FP64 (``t* > tol``, batched_simplex.cu phase 2).

Checked record by record against the oracle on instances whose sets reach
that case (small n, ill-conditioned square KKT blocks, and the m = 62
instance): the same feasible, optimal and region sets with bit-identical t*
and r* for every optimal set; every set the check settled is not optimal for
the oracle, its bound is negative and at least the oracle's FP64 LP2 optimum
(weak duality); and the per-instance counter equals the records.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = {
    "member30-n6m34p5": (lambda: P.batch_member(30), 6),
    "member11-n6m27p5": (lambda: P.batch_member(11), 6),
    "member14-n6m70p5-k4": (lambda: P.batch_member(14), 4),
    "m62-k4": (lambda: P.random_n12_m62_p6(), 4),
}
FP64_LP2, CERT_LP2 = 2, 8


def _sorted(rec):
    rec = rec[rec["level"] >= 0]
    return rec[np.lexsort([rec["mask_lo"], rec["mask_hi"]])]


def _same(a, b):
    return np.array_equal(np.nan_to_num(a, nan=12345.0), np.nan_to_num(b, nan=12345.0))


@pytest.mark.parametrize("case", list(CASES))
def test_fp64_check_of_the_fp32_dual_basis(gpu_lib, case):
    make, kmax = CASES[case]
    prob = P.scale_problem(make())
    ref = O.enumerate_sets(prob, k_max=kmax, nthreads=8)
    res = solver.solve([prob], precision=solver.MIXED, k_max=kmax, record=1, rec_cap=ref.n_cand + 16,
                       cand_cap=ref.n_cand + 1024, arena_bytes=1 << 30)
    assert res.status == 0 and res.overflow == 0
    g, o = _sorted(res.rec), _sorted(ref.cand)
    assert np.array_equal(g["mask_lo"], o["mask_lo"]) and np.array_equal(g["mask_hi"], o["mask_hi"])
    for f in ("feasible", "optimal", "region"):
        assert np.array_equal(g[f], o[f]), (f, int(np.sum(g[f] != o[f])))
    opt = o["optimal"] == 1
    assert _same(g["t"][opt], o["t"][opt]) and _same(g["r"][opt], o["r"][opt])
    cert = (g["fp64"] & CERT_LP2) != 0
    assert np.all((g["fp64"][cert] & FP64_LP2) != 0)
    assert not np.any(o["optimal"][cert])
    bound, t64 = g["t"][cert], o["t"][cert]
    assert np.all(bound < 0.0)
    # weak duality: the bound is at least the FP64 LP2 optimum of the same rows
    assert np.all(bound >= t64 - 1e-9 * np.maximum(1.0, np.abs(t64))), float(np.max(t64 - bound))
    assert res.total("lp2_certified") == int(cert.sum())
    assert res.total("lp2_certified") <= res.total("fallback_opt")
    print(case, "feasible", ref.n_feasible, "optimal", ref.n_optimal, "FP64 optimality evaluations",
          res.total("fallback_opt"), "settled by the basis check", int(cert.sum()))


def test_basis_check_on_the_batch_members(gpu_lib):
    """The three members with the most FP64 evaluations, as one batch: the
    check settles sets, and the verdicts equal the FP64 path's."""
    probs = [P.scale_problem(P.batch_member(s)) for s in (11, 23, 30)]
    kw = dict(k_max=[p.n for p in probs], budget=1 << 19, cand_cap=1 << 21, arena_bytes=1 << 30)
    a = solver.solve(probs, precision=solver.FP64, **kw)
    b = solver.solve(probs, precision=solver.MIXED, **kw)
    assert a.status == b.status == 0
    for f in ("candidates", "feasible", "optimal", "regions", "feasible_digest", "optimal_digest", "region_digest"):
        assert np.array_equal(a.inst[f], b.inst[f]), f
    assert b.total("lp2_certified") > 0
    ka = np.lexsort([a.opt["mask_lo"], a.opt["mask_hi"], a.opt["inst"]])
    kb = np.lexsort([b.opt["mask_lo"], b.opt["mask_hi"], b.opt["inst"]])
    assert _same(a.opt["t"][ka], b.opt["t"][kb]) and _same(a.opt["r"][ka], b.opt["r"][kb])
    print("members 11, 23, 30: FP64 optimality evaluations", b.total("fallback_opt"), "settled by the basis check",
          b.total("lp2_certified"), "optimal", b.total("optimal"))
