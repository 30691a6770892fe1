"""Limits of the device path.

* m = 128, the largest instance the 128-bit active-set masks hold: every
  candidate with |S| <= 3 bit-identical to the oracle in FP64 (constraint 127
  included), the same verdicts in mixed precision.  Its 132 rows also exceed
  the 96-row limit of the register-bookkeeping simplex and of the dual bound,
  so the generic FP32 paths run.
* m = 129 and an empty instance list are rejected with MPQP_EINVAL.
* k_min > 0: lower levels are enumerated for pruning but not evaluated; the
  evaluated sets match the oracle's.
* The optimal sets come back ordered by instance, then size, then the sorted
  element lists (also for masks that use the high word), and equal the
  oracle's.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _sorted(rec):
    rec = rec[rec["level"] >= 0]
    return rec[np.lexsort([rec["mask_lo"], rec["mask_hi"]])]


def test_m128_bit_exact_and_mixed(gpu_lib):
    prob = P.scale_problem(P.random_mpqp(3, 128, 2, seed=7))
    ref = O.enumerate_sets(prob, k_max=3, nthreads=8)
    kw = dict(k_max=3, record=1, rec_cap=ref.n_cand + 16, cand_cap=1 << 20, arena_bytes=1 << 28)
    r64 = solver.solve([prob], precision=solver.FP64, **kw)
    r32 = solver.solve([prob], precision=solver.MIXED, **kw)
    assert r64.status == 0 and r32.status == 0 and r64.candidates == ref.n_cand
    g, o, h = _sorted(r64.rec), _sorted(ref.cand), _sorted(r32.rec)
    assert np.any(g["mask_hi"] >> np.uint64(63) & np.uint64(1))      # constraint 127 appears
    for f in ("mask_lo", "mask_hi", "lp1_pivots", "feasible", "optimal", "region", "lp2_pivots"):
        assert np.array_equal(g[f], o[f]), f
    assert np.array_equal(g["z"], o["z"])
    for f in ("feasible", "optimal", "region"):
        assert np.array_equal(h[f], o[f]), f


def test_m129_and_empty_batch_are_rejected(gpu_lib):
    prob = P.scale_problem(P.random_mpqp(3, 129, 2, seed=7))
    with pytest.raises(solver.MpqpError) as e:
        solver.solve([prob], precision=solver.FP64, k_max=1)
    assert e.value.code == solver.EINVAL
    with pytest.raises(solver.MpqpError) as e:
        solver.solve([], precision=solver.FP64)
    assert e.value.code == solver.EINVAL


@pytest.mark.parametrize("precision", [solver.FP64, solver.MIXED])
def test_k_min_evaluates_only_upper_levels(gpu_lib, precision):
    prob = P.scale_problem(P.random_n10_m43_p4())
    ref = O.enumerate_sets(prob, k_min=2, k_max=3, nthreads=8)
    res = solver.solve([prob], precision=precision, k_min=2, k_max=3, cand_cap=1 << 18, arena_bytes=1 << 28)
    assert res.status == 0
    assert res.candidates == ref.n_cand and res.total("feasible") == ref.n_feasible
    assert res.total("optimal") == ref.n_optimal and res.total("regions") == ref.n_region
    assert all(int(o["level"]) >= 2 for o in res.opt)


def test_optimal_sets_in_instance_level_lexicographic_order(gpu_lib):
    probs = [P.scale_problem(P.random_mpqp(3, 128, 2, seed=7)), P.scale_problem(P.random_n4_m10_p2()),
             P.scale_problem(P.random_mpqp(5, 70, 3, seed=3))]
    res = solver.solve(probs, precision=solver.MIXED, k_max=3, cand_cap=1 << 20, arena_bytes=1 << 28)
    assert res.status == 0 and len(res.opt) > 0
    keys = [(int(o["inst"]), int(o["level"]), tuple(solver.mask_to_set(o["mask_lo"], o["mask_hi"]))) for o in res.opt]
    assert all(len(k[2]) == k[1] for k in keys)
    assert all(a < b for a, b in zip(keys, keys[1:]))
    assert any(max(k[2]) >= 64 for k in keys if k[2])                      # high-word masks are ordered too
    for i, prob in enumerate(probs):
        ref = O.enumerate_sets(prob, k_max=3, nthreads=8)
        want = sorted((c["level"], tuple(O.mask_to_set(c["mask_lo"], c["mask_hi"]))) for c in ref.cand if c["optimal"])
        assert [(k[1], k[2]) for k in keys if k[0] == i] == want, i
