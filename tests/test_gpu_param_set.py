"""Parameter sets that are not a box.

The FP32 screens bound theta by the box (the reach of each parameter), so an
instance whose parameter set has any other row takes the primal route and has
every optimality verdict decided in FP64; its LP1 still runs in FP32 with the
FP64 certificates.  Here the box gains a cut (theta_1 + theta_2 <= 1.2), for
an mpQP and an mpLP: every candidate's feasible, optimal and region verdict,
and the FP64 t* and r* of every optimal set, must equal the oracle's in both
precisions.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _with_cut(prob):
    p = prob.CRA.shape[1]
    cut = np.zeros((1, p))
    cut[0, 0] = cut[0, 1] = 1.0
    CRA = np.vstack([prob.CRA, cut])
    CRb = np.concatenate([np.asarray(prob.CRb).ravel(), [1.2]])
    return P.MPQP(prob.Q, prob.c, prob.H, prob.A, prob.b, prob.F, CRA, CRb, name=prob.name + "+cut")


CASES = {
    "mpqp-n6m20p3": (lambda: P.random_mpqp(6, 20, 3, seed=7), 6),
    "mpqp-n10m43p4-k3": (lambda: P.random_n10_m43_p4(), 3),
    "mplp-n5m16p3": (lambda: P.random_mplp(5, 16, 3, seed=8), 5),
}


def _sorted(rec):
    rec = rec[rec["level"] >= 0]
    return rec[np.lexsort([rec["mask_lo"], rec["mask_hi"]])]


def _same(a, b):
    return np.array_equal(np.nan_to_num(a, nan=12345.0), np.nan_to_num(b, nan=12345.0))


@pytest.mark.parametrize("precision", [solver.FP64, solver.MIXED])
@pytest.mark.parametrize("case", list(CASES))
def test_non_box_parameter_set_matches_oracle(gpu_lib, case, precision):
    make, kmax = CASES[case]
    prob = P.scale_problem(_with_cut(make()))
    ref = O.enumerate_sets(prob, k_max=kmax, nthreads=8)
    res = solver.solve([prob], precision=precision, k_max=kmax, record=1, rec_cap=ref.n_cand + 16,
                       cand_cap=max(4096, ref.n_cand + 1024), arena_bytes=1 << 28)
    assert res.status == 0 and res.overflow == 0
    g, o = _sorted(res.rec), _sorted(ref.cand)
    assert np.array_equal(g["mask_lo"], o["mask_lo"]) and np.array_equal(g["mask_hi"], o["mask_hi"])
    for f in ("feasible", "optimal", "region"):
        assert np.array_equal(g[f], o[f]), (f, int(np.sum(g[f] != o[f])))
    opt = o["optimal"] == 1
    assert _same(g["t"][opt], o["t"][opt]) and _same(g["r"][opt], o["r"][opt])
    assert res.total("regions") == ref.n_region
    if precision == solver.MIXED:
        # no box: no FP32 "not optimal"; every feasible set is decided in FP64
        feas = (g["feasible"] == 1) & (g["level"] >= 1)
        assert np.all((g["fp64"][feas] & 2) != 0)
        assert res.total("lp2_first_stage_lps") == 0
    print(case, "precision", precision, "candidates", ref.n_cand, "feasible", ref.n_feasible, "optimal",
          ref.n_optimal, "regions", ref.n_region)
