"""FP32 LP1 "infeasible" verdicts rest on an FP64 dual certificate.

Mixed precision solves LP1 in FP32.  A candidate is infeasible only when the
FP64 dual certificate built from its final FP32 basis (``k_lp1_cert``)
proves ``z* >= beta.y / s > tol_feas``; every other candidate without a
certified-feasible basis is re-solved in FP64 (``k_lp1_fp64``).  The
reference decides LP1 in FP64 (``|z| <= tol``, batched_simplex.cu:308-314).

Checked record by record on the five workloads at |S| <= 3 (|S| <= 4 on the
smallest): every infeasible verdict carries either the certificate bit or the
FP64 re-solve bit; each certified bound lies in (tol_feas, z*] with z* the
oracle's FP64 LP1 optimum of the same set (weak duality); the oracle's own
chain finds the same sets infeasible (and its own certificate, where its
final basis gives one, proves them); the per-instance counters equal the
record counts.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = {
    "n4m10p2": (lambda: P.random_n4_m10_p2(), 4),
    "n10m43p4-k3": (lambda: P.random_n10_m43_p4(), 3),
    "m62-k3": (lambda: P.random_n12_m62_p6(), 3),
    "illcond-k3": (lambda: P.illcond_n16_m62_p8(), 3),
    "mpc-k3": (lambda: P.mpc_mpqp(0), 3),
    "n5m14p2-k5": (lambda: P.random_mpqp(5, 14, 2, seed=13), 5),
}

CERT, RESOLVED = 4, 1


def _sorted(rec):
    rec = rec[rec["level"] >= 1]
    return rec[np.lexsort([rec["mask_lo"], rec["mask_hi"]])]


@pytest.mark.parametrize("case", list(CASES))
def test_fp32_infeasible_verdicts_are_certified_or_resolved(gpu_lib, case):
    make, kmax = CASES[case]
    prob = P.scale_problem(make())
    ref = O.enumerate_sets(prob, k_max=kmax, nthreads=4)
    res = solver.solve([prob], precision=solver.MIXED, k_max=kmax, record=1, rec_cap=ref.n_cand + 16,
                       cand_cap=max(4096, ref.n_cand), arena_bytes=1 << 28)
    assert res.status == 0 and res.overflow == 0
    g, o = _sorted(res.rec), _sorted(ref.cand)
    assert len(g) == len(o)
    assert np.array_equal(g["mask_lo"], o["mask_lo"]) and np.array_equal(g["mask_hi"], o["mask_hi"])
    assert np.array_equal(g["feasible"], o["feasible"])
    tol_feas = O.default_tol().tol_feas
    cert = (g["fp64"] & CERT) != 0
    resolved = (g["fp64"] & RESOLVED) != 0
    infeasible = g["feasible"] == 0
    # no FP32 infeasible verdict without an FP64 proof or an FP64 solve
    assert np.all(cert[infeasible] | resolved[infeasible])
    assert not np.any(cert & resolved)
    assert not np.any(cert & ~infeasible)
    bound = g["lp1_bound"][cert]
    assert np.all(bound > tol_feas)
    # weak duality against the oracle's FP64 optimum of the same LP
    z = o["z"][cert]
    assert np.all(bound <= z * (1 + 1e-9) + 1e-12), float(np.max(bound - z))
    # the oracle's FP64 chain finds these sets infeasible, and where its own
    # final basis gives a certificate (every free variable basic) it proves
    # them too
    idx = np.nonzero(cert)[0]
    rng = np.random.default_rng(1)
    for i in idx[rng.permutation(len(idx))[:200]]:
        S = O.mask_to_set(g["mask_lo"][i], g["mask_hi"][i])
        ok, b64, z64, used = O.lp1_dual_bound(prob, S)
        assert used == len(S) and z64 > tol_feas, (S, z64)
        assert not ok or b64 > tol_feas, (S, b64, z64)
    assert res.total("lp1_certified") == int(cert.sum())
    assert res.total("fallback_lp1") == int(resolved.sum())
    assert res.total("lp1_cert_missed") <= res.total("fallback_lp1")
    print(case, "infeasible", int(infeasible.sum()), "certified", int(cert.sum()), "re-solved",
          int(resolved.sum()), "cert missed", res.total("lp1_cert_missed"), "free-variable misses",
          res.total("lp1_cert_freevar"))


VERTEX = 16


@pytest.mark.parametrize("case", ["m62-k4", "n10m43p4-k4"])
def test_fp64_vertex_check_of_last_level_optima(gpu_lib, case):
    """At an instance's last level, an FP32 LP1 optimum with every slack of S'
    nonbasic and a smallest basic slack inside the FP32 margin is decided by
    the FP64 vertex check of its final basis instead of an FP64 re-solve:
    every set it accepts is feasible for the oracle, lies at the last level,
    and carries a positive smallest slack; the counter equals the records."""
    make = {"m62-k4": P.random_n12_m62_p6, "n10m43p4-k4": P.random_n10_m43_p4}[case]
    kmax = 4
    prob = P.scale_problem(make())
    ref = O.enumerate_sets(prob, k_max=kmax, nthreads=8)
    res = solver.solve([prob], precision=solver.MIXED, k_max=kmax, record=1, rec_cap=ref.n_cand + 16,
                       cand_cap=ref.n_cand + 1024, arena_bytes=1 << 29)
    assert res.status == 0 and res.overflow == 0
    g, o = _sorted(res.rec), _sorted(ref.cand)
    assert np.array_equal(g["mask_lo"], o["mask_lo"]) and np.array_equal(g["mask_hi"], o["mask_hi"])
    assert np.array_equal(g["feasible"], o["feasible"])
    vtx = (g["fp64"] & VERTEX) != 0
    assert np.all(o["feasible"][vtx] == 1)
    assert np.all(g["level"][vtx] == kmax)
    assert np.all(g["lp1_bound"][vtx] > 0.0)
    assert not np.any(vtx & ((g["fp64"] & (CERT | RESOLVED)) != 0))
    assert res.total("lp1_vertex_checked") == int(vtx.sum()) > 0
    print(case, "vertex checks", int(vtx.sum()), "FP64 re-solves", res.total("fallback_lp1"))
