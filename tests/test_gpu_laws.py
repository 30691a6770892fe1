"""Region laws on the device (FP64) against the oracle and the reference math.

The affine laws lambda(theta), x(theta) and the normalised region rows of
every region found are compared with
* the C oracle (same operation order: identical to 1e-12 relative), and
* a line-by-line restatement of ``compute_critical_region`` (numpy pinv,
  utils.py:23-97): within 1e-8 relative, as the target requires.  Rows whose
  theta part vanishes up to rounding are dropped by the relative test both
  sides use (max|g| <= 1e-12 max(1,|h|)) instead of the exact-zero test.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O
from oracle import reference_lp as R

pytestmark = pytest.mark.gpu

CASES = {
    "n4m10p2": (lambda: P.random_n4_m10_p2(), 4),
    "n10m43p4-k3": (lambda: P.random_n10_m43_p4(), 3),
    "m62-k2": (lambda: P.random_n12_m62_p6(), 2),
    "mpc-k3": (lambda: P.mpc_mpqp(0), 3),
}


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    if a.shape != b.shape:
        return np.inf
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("case", list(CASES))
def test_region_laws_match_oracle_and_reference(gpu_lib, case):
    make, kmax = CASES[case]
    prob = P.scale_problem(make())
    res = solver.solve([prob], precision=solver.FP64, k_max=kmax, cand_cap=1 << 18, arena_bytes=1 << 28)
    regions = [solver.mask_to_set(o["mask_lo"], o["mask_hi"]) for o in res.opt if o["region"]]
    assert regions, "no region found"
    sets = regions[:200]
    laws = solver.region_laws(prob, sets)
    worst_ref = 0.0
    for S, law in zip(sets, laws):
        assert law is not None
        rec, ol = O.check_set(prob, S, want_laws=True)
        assert rec["region"] == 1
        for key in ("lagrange_A", "lagrange_b", "parameter_A", "parameter_b", "CR_As", "CR_bs"):
            assert _rel(law[key], ol[key]) <= 1e-12, (S, key)
        reg, r = R.region_for(prob, S, zero_tol=1e-12)
        assert reg is not None
        # 1e-8 relative per entry with a 1e-12 absolute floor
        for key in ("lagrange_A", "parameter_A", "CR_As", "lagrange_b", "parameter_b", "CR_bs"):
            b = np.asarray(reg[key]).reshape(np.shape(law[key]))
            assert np.allclose(law[key], b, rtol=1e-8, atol=1e-12), (S, key)
            worst_ref = max(worst_ref, float(np.max(np.abs(law[key] - b) / (np.abs(b) + 1e-4))) if b.size else 0.0)
        assert abs(rec["r"] - r) <= 1e-8 * max(1.0, abs(r)), (S, rec["r"], r)


def test_region_laws_reject_bad_sets(gpu_lib):
    prob = P.scale_problem(P.random_n4_m10_p2())
    with pytest.raises(solver.MpqpError):
        solver.region_laws(prob, [[0, 1, 2, 3, 4]])        # |S| > n
    with pytest.raises(solver.MpqpError):
        solver.region_laws(prob, [[prob.m]])               # index out of range


ERR_CASES = {
    "m62-k3": (lambda: P.random_n12_m62_p6(), 3),
    "illcond-k3": (lambda: P.illcond_n16_m62_p8(), 3),
    "mpc-k3": (lambda: P.mpc_mpqp(0), 3),
    "mplp-n5": (lambda: P.random_mplp(5, 16, 3, seed=2), 5),
}


@pytest.mark.parametrize("case", list(ERR_CASES))
def test_every_result_states_its_error(gpu_lib, case):
    """Each optimal set carries the stated relative error of its laws (one
    FP64 iterative-refinement step of its KKT solve, mpqp_opt_set.err), in
    both precisions and identical between them; mpqp_critical_regions states
    the same error beside the laws.  The stated error is a sound estimate:
    the laws' actual deviation from an independent numpy restatement of
    utils.py:25-36 stays within max(1e3 x err, 1e-12), and every region here
    states an error below the 1e-8 target."""
    make, kmax = ERR_CASES[case]
    prob = P.scale_problem(make())
    kw = dict(k_max=kmax, cand_cap=1 << 20, arena_bytes=1 << 28)
    r64 = solver.solve([prob], precision=solver.FP64, **kw)
    r32 = solver.solve([prob], precision=solver.MIXED, **kw)
    assert r64.status == 0 and r32.status == 0
    key = lambda r: {(int(o["mask_lo"]), int(o["mask_hi"])): float(o["err"]) for o in r.opt}
    e64, e32 = key(r64), key(r32)
    assert e64.keys() == e32.keys() and e64
    for k in e64:
        assert e64[k] == e32[k] or (np.isnan(e64[k]) and np.isnan(e32[k])), k
    # every optimal set states a finite error, except an mpLP set with
    # |S| < n (no unique law: never a region)
    errs = np.array(list(e64.values()))
    short = np.array([len(solver.mask_to_set(*k)) < prob.n for k in e64]) if not prob.Q.any() else 0
    assert np.all(np.isfinite(errs) | short) and np.all(errs[np.isfinite(errs)] >= 0)
    errs = errs[np.isfinite(errs)]
    regions = [o for o in r64.opt if o["region"]]
    assert regions and max(float(o["err"]) for o in regions) < 1e-8
    sets = [solver.mask_to_set(o["mask_lo"], o["mask_hi"]) for o in regions[:100]]
    laws = solver.region_laws(prob, sets, with_radius=True)
    for o, S, law in zip(regions[:100], sets, laws):
        assert law is not None and law["err"] == float(o["err"]) and law["r"] == float(o["r"]), S
        if prob.Q.any():
            reg, _ = R.region_for(prob, S, zero_tol=1e-12)
            dev = _rel(law["lagrange_A"], reg["lagrange_A"])
            assert dev <= max(1e3 * law["err"], 1e-12), (S, dev, law["err"])
    print(case, "optimal sets", len(errs), "max stated error", float(errs.max()),
          "median", float(np.median(errs)))
