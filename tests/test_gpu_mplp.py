"""mpLP instances (Q = 0) on the device against the oracle.

* FP64 kernels: every checked candidate's LP values, pivot counts and
  verdicts are bit-identical to the oracle's mpLP path (which
  tests/test_oracle_mplp.py pins to the reference's LP2 solved by HiGHS).
* Mixed precision: the feasible, optimal and region sets equal the FP64
  path's.  LP1 runs in FP32; at |S| <= 6 the FP32 first stage proves sets
  not optimal from their multiplier rows (-Psi(theta)) and the parameter
  box, and every set it leaves is decided in FP64.
* A batch mixing mpQP and mpLP instances gives each instance the sets it
  gets alone (the two kinds run in separate optimality kernels).
* Region laws of mpLP regions match the oracle's; a set with |S| < n has no
  unique law and is reported as such.
* The reference's C-ABI entry point reads Q = 0 back from the LP matrices
  and returns the oracle's optimal sets.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import host
from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = {
    "n3m10p2-h0-exhaustive": (lambda: P.random_mplp(3, 10, 2, seed=0, h_scale=0.0), 3, True),
    "n3m10p2-h1-exhaustive": (lambda: P.random_mplp(3, 10, 2, seed=1, h_scale=1.0), 3, True),
    "n6m24p3-h1": (lambda: P.random_mplp(6, 24, 3, seed=2, h_scale=1.0), 6, False),
    "n6m20p3-h1": (lambda: P.random_mplp(6, 20, 3, seed=3, h_scale=1.0), 6, False),
    "n7m22p3-h0": (lambda: P.random_mplp(7, 22, 3, seed=4, h_scale=0.0), 7, False),
    "n7m22p3-h1": (lambda: P.random_mplp(7, 22, 3, seed=4, h_scale=1.0), 7, False),
}


def _sorted(rec):
    rec = rec[rec["level"] >= 0]
    return rec[np.lexsort([rec["mask_lo"], rec["mask_hi"]])]


def _same(a, b):
    return np.array_equal(np.nan_to_num(a, nan=12345.0), np.nan_to_num(b, nan=12345.0))


@pytest.mark.parametrize("case", list(CASES))
def test_mplp_fp64_bit_exact_vs_oracle(gpu_lib, case):
    make, kmax, exh = CASES[case]
    prob = P.scale_problem(make())
    ref = O.enumerate_sets(prob, k_max=kmax, exhaustive=exh, nthreads=4)
    res = solver.solve([prob], precision=solver.FP64, k_max=kmax, exhaustive=int(exh), record=1,
                       rec_cap=ref.n_cand + 16, cand_cap=max(4096, ref.n_cand), arena_bytes=1 << 28)
    assert res.status == 0 and res.overflow == 0
    g, o = _sorted(res.rec), _sorted(ref.cand)
    assert len(g) == len(o) == ref.n_cand
    assert np.array_equal(g["mask_lo"], o["mask_lo"]) and np.array_equal(g["mask_hi"], o["mask_hi"])
    for f in ("level", "lp1_status", "lp1_pivots", "feasible", "optimal", "region", "lp2_status", "lp2_pivots",
              "cheb_pivots"):
        assert np.array_equal(g[f], o[f]), f
    for f in ("z", "t", "r"):
        assert _same(g[f], o[f]), f
    assert res.total("optimal") == ref.n_optimal == len(res.opt)
    assert res.total("regions") == ref.n_region > 0
    # sets with |S| < n: LP2 decided through the two-phase LP, never regions
    short = (o["feasible"] == 1) & (o["level"] < prob.n)
    assert np.all(o["region"][short] == 0)
    assert np.any(o["lp2_status"][short] == O.INFEASIBLE)


@pytest.mark.parametrize("case", list(CASES))
def test_mplp_mixed_same_sets_as_fp64(gpu_lib, case):
    make, kmax, exh = CASES[case]
    prob = P.scale_problem(make())
    a = solver.solve([prob], precision=solver.FP64, k_max=kmax, exhaustive=int(exh))
    b = solver.solve([prob], precision=solver.MIXED, k_max=kmax, exhaustive=int(exh))
    assert a.status == b.status == 0
    for f in ("feasible_digest", "optimal_digest", "region_digest", "feasible", "optimal", "regions", "candidates"):
        assert a.inst[0][f] == b.inst[0][f], f
    # the FP32 first stage settles some sets; the rest go to the FP64 kernels
    assert 0 < b.inst[0]["fallback_opt"] < b.inst[0]["feasible"], (b.inst[0]["fallback_opt"], b.inst[0]["feasible"])
    assert b.inst[0]["lp2_first_stage_lps"] > 0


@pytest.mark.parametrize("tile_w", [8, 16, 32])
def test_mplp_first_stage_above_six(gpu_lib, tile_w):
    """The sets with |S| > 6 of an mpLP over a box take the first stage one
    set per tile (k_opt_screen_tiles, the multiplier rows -Psi and the box):
    with the checks confined to |S| = 7, 8 it runs LPs, settles some sets,
    and the verdicts stay those of the FP64 path."""
    prob = P.scale_problem(P.random_mplp(8, 24, 3, seed=6))
    a = solver.solve([prob], precision=solver.FP64, k_min=7, k_max=8)
    b = solver.solve([prob], precision=solver.MIXED, k_min=7, k_max=8, tile_w=tile_w)
    assert a.status == b.status == 0
    for f in ("feasible_digest", "optimal_digest", "region_digest", "feasible", "optimal", "regions", "candidates"):
        assert a.inst[0][f] == b.inst[0][f], f
    lps, fb = b.inst[0]["lp2_first_stage_lps"], b.inst[0]["fallback_opt"]
    assert lps > 0 and fb < lps, (lps, fb)
    print("tile", tile_w, "first-stage LPs", lps, "FP64 fallbacks", fb, "optimal", b.inst[0]["optimal"])


def test_mplp_second_stage_and_basis_check(gpu_lib):
    """mpLP sets with |S| = n that the first stage leaves take the dual
    route's second stage (multiplier rows from Psi, region rows from Gamma),
    and those whose FP32 bound is negative but inside its margin the FP64
    check of their dual basis: on eight instances of the mpLP batch the
    verdicts equal the FP64 path's and the check settles sets."""
    probs = [P.scale_problem(p) for p in P.mplp_batch()[:8]]
    a = solver.solve(probs, precision=solver.FP64)
    b = solver.solve(probs, precision=solver.MIXED)
    assert a.status == b.status == 0
    for f in ("feasible_digest", "optimal_digest", "region_digest", "feasible", "optimal", "regions", "candidates"):
        assert np.array_equal(a.inst[f], b.inst[f]), f
    ka = np.lexsort([a.opt["mask_lo"], a.opt["mask_hi"], a.opt["inst"]])
    kb = np.lexsort([b.opt["mask_lo"], b.opt["mask_hi"], b.opt["inst"]])
    assert _same(a.opt["t"][ka], b.opt["t"][kb]) and _same(a.opt["r"][ka], b.opt["r"][kb])
    assert b.total("lp2_certified") > 0
    print("mpLP batch (8): FP64 optimality evaluations", b.total("fallback_opt"), "settled by the basis check",
          b.total("lp2_certified"), "of", b.total("feasible"), "feasible sets")


@pytest.mark.parametrize("precision", [solver.FP64, solver.MIXED])
def test_batch_of_mpqp_and_mplp_instances(gpu_lib, precision):
    probs = [P.scale_problem(p) for p in (P.random_n4_m10_p2(), P.random_mplp(6, 24, 3, seed=2),
                                          P.random_mpqp(5, 14, 2, seed=13), P.random_mplp(3, 10, 2, seed=0,
                                                                                         h_scale=0.0))]
    batch = solver.solve(probs, precision=precision, k_max=4)
    assert batch.status == 0
    for i, prob in enumerate(probs):
        solo = solver.solve([prob], precision=precision, k_max=4)
        for f in ("feasible_digest", "optimal_digest", "region_digest", "candidates", "optimal", "regions"):
            assert batch.inst[i][f] == solo.inst[0][f], (i, f)


def test_mplp_region_laws_match_oracle(gpu_lib):
    prob = P.scale_problem(P.random_mplp(6, 24, 3, seed=2))
    res = solver.solve([prob], precision=solver.FP64, k_max=prob.n)
    regions = [solver.mask_to_set(o["mask_lo"], o["mask_hi"]) for o in res.opt if o["region"]]
    short = [solver.mask_to_set(o["mask_lo"], o["mask_hi"]) for o in res.opt if o["level"] < prob.n]
    assert regions and short
    laws = solver.region_laws(prob, regions + short[:5])
    for S, law in zip(regions, laws):
        rec, ol = O.check_set(prob, S, want_laws=True)
        assert rec["region"] == 1 and law is not None
        for key in ("lagrange_A", "lagrange_b", "parameter_A", "parameter_b", "CR_As", "CR_bs"):
            want = np.asarray(ol[key])
            assert np.shape(law[key]) == want.shape, key
            if want.size:
                assert np.max(np.abs(law[key] - want)) <= 1e-12 * max(np.max(np.abs(want)), 1e-300), (S, key)
    assert all(law is None for law in laws[len(regions):])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_abi_with_zero_q(gpu_lib, precision, monkeypatch):
    monkeypatch.setenv("MPQP_PRECISION", precision)
    lib = host.load_mpqp_cuda()
    lib.warm_up()
    prog = host.MPQPProb.from_mpqp(P.random_mplp(4, 13, 3, seed=5))
    prog.process_constraints(scale_method=1)
    d = host.build_lp_data(prog)
    r = host.call_mpqp(lib, d)
    g = r.contents
    assert g.status == 0, solver.last_error()
    e = O.enumerate_sets(prog.to_mpqp(), k_max=d["num_x"])
    sets = host.decode_active_sets(g.active_sets, g.n_final_lps, d["num_x"])
    want = sorted(O.mask_to_set(c["mask_lo"], c["mask_hi"]) for c in e.cand if c["optimal"])
    assert sorted(sets) == want and want
    assert g.n_regions == e.n_region > 0
    lib.mpqp_free(r)
