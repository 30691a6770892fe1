"""GPU parity: the device kernels against the CPU oracle (through the C ABI).

* FP64 kernels: every checked candidate, its LP values (z, t*, r*), pivot
  counts and verdicts are bit-identical to the oracle's.
* Mixed precision (FP32 pivots + FP64 certificates): the feasible, optimal
  and region sets are identical to the FP64 path's.
"""
import os

import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = {
    "n4m10p2": (lambda: P.random_n4_m10_p2(), 4, False),
    "n4m10p2-exhaustive": (lambda: P.random_n4_m10_p2(), 4, True),
    "n10m43p4-k3": (lambda: P.random_n10_m43_p4(), 3, False),
    "m62-k3": (lambda: P.random_n12_m62_p6(), 3, False),
    "illcond-k3": (lambda: P.illcond_n16_m62_p8(), 3, False),
    "mpc-k3": (lambda: P.mpc_mpqp(0), 3, False),
}


def _sorted(rec, key_inst=False):
    rec = rec[rec["level"] >= 0]
    keys = [rec["mask_lo"], rec["mask_hi"]] + ([rec["inst"]] if key_inst else [])
    return rec[np.lexsort(keys)]


def _same(a, b):
    return np.array_equal(a, b) or np.array_equal(np.nan_to_num(a, nan=12345.0), np.nan_to_num(b, nan=12345.0))


def _fp64_records_equal_oracle(res, ref):
    assert res.status == 0 and res.overflow == 0
    assert res.candidates == ref.n_cand
    g = _sorted(res.rec)
    o = _sorted(ref.cand)
    assert len(g) == len(o) == ref.n_cand
    assert np.array_equal(g["mask_lo"], o["mask_lo"]) and np.array_equal(g["mask_hi"], o["mask_hi"])
    for f in ("level", "lp1_status", "lp1_pivots", "feasible", "optimal", "region", "lp2_pivots", "cheb_pivots"):
        assert np.array_equal(g[f], o[f]), f
    for f in ("z", "t", "r"):
        assert _same(g[f], o[f]), f
    fe = o["feasible"] == 1
    assert np.array_equal(g["licq"][fe], o["licq"][fe])
    assert res.total("feasible") == ref.n_feasible
    assert res.total("optimal") == ref.n_optimal == len(res.opt)
    assert res.total("regions") == ref.n_region
    assert res.total("pruned") == ref.n_pruned
    return g, o


@pytest.mark.parametrize("case", list(CASES))
def test_fp64_bit_exact_vs_oracle(gpu_lib, case):
    make, kmax, exh = CASES[case]
    prob = P.scale_problem(make())
    ref = O.enumerate_sets(prob, k_max=kmax, exhaustive=exh, nthreads=4)
    res = solver.solve([prob], precision=solver.FP64, k_max=kmax, exhaustive=int(exh), record=1,
                       rec_cap=ref.n_cand + 16, cand_cap=max(4096, ref.n_cand), arena_bytes=1 << 28)
    _fp64_records_equal_oracle(res, ref)


DEEP = {
    "m62-k5": (lambda: P.random_n12_m62_p6(), 5),      # 6.6M candidates
    "mpc-k4": (lambda: P.mpc_mpqp(0), 4),
    "illcond-k4": (lambda: P.illcond_n16_m62_p8(), 4),
}


@pytest.mark.parametrize("case", list(DEEP))
def test_deep_levels_vs_oracle(gpu_lib, case):
    """Record-level parity at the deep levels: the FP64 kernels bit-identical
    to the oracle on every checked candidate, and the mixed path's feasible,
    optimal and region verdicts -- with the FP64 t* and r* of every optimal
    set -- equal to the oracle's."""
    make, kmax = DEEP[case]
    prob = P.scale_problem(make())
    ref = O.enumerate_sets(prob, k_max=kmax, nthreads=os.cpu_count() or 4)
    kw = dict(k_max=kmax, record=1, rec_cap=ref.n_cand + 16, cand_cap=ref.n_cand + 1024, mem_fraction=0.5)
    r64 = solver.solve([prob], precision=solver.FP64, **kw)
    _, o = _fp64_records_equal_oracle(r64, ref)
    del r64
    r32 = solver.solve([prob], precision=solver.MIXED, **kw)
    assert r32.status == 0 and r32.overflow == 0
    g = _sorted(r32.rec)
    assert np.array_equal(g["mask_lo"], o["mask_lo"]) and np.array_equal(g["mask_hi"], o["mask_hi"])
    for f in ("feasible", "optimal", "region"):
        assert np.array_equal(g[f], o[f]), (f, int(np.sum(g[f] != o[f])))
    opt = o["optimal"] == 1
    assert _same(g["t"][opt], o["t"][opt]) and _same(g["r"][opt], o["r"][opt])
    print(case, "candidates", ref.n_cand, "feasible", ref.n_feasible, "optimal", ref.n_optimal,
          "certified infeasible", r32.total("lp1_certified"), "FP64 re-solves", r32.total("fallback_lp1"))


def test_level6_sample_vs_oracle(gpu_lib):
    """The bench's depth (|S| <= 6 on the m = 62 instance, 54.3M candidates)
    in mixed precision, sampled against the oracle (each set's warm-start
    chain replayed in FP64): a seeded sample of the level-6 optimal sets keeps
    the oracle's verdicts and bit-identical t* and r*; a seeded sample of
    random 6-sets is optimal for the oracle exactly when the device lists it."""
    prob = P.scale_problem(P.random_n12_m62_p6())
    r32 = solver.solve([prob], precision=solver.MIXED, k_max=6, mem_fraction=0.8)
    assert r32.status == 0
    opt6 = r32.opt[r32.opt["level"] == 6]
    assert len(opt6) > 1000
    listed = {(int(a), int(b)) for a, b in zip(r32.opt["mask_lo"], r32.opt["mask_hi"])}
    rng = np.random.default_rng(6)
    for row in opt6[rng.permutation(len(opt6))[:1500]]:
        S = O.mask_to_set(row["mask_lo"], row["mask_hi"])
        d, _ = O.check_set(prob, S)
        assert d["feasible"] == 1 and d["optimal"] == 1, S
        assert d["t"] == row["t"] and d["r"] == row["r"] and d["region"] == row["region"], S
    hits = 0
    for _ in range(3000):
        S = sorted(rng.choice(prob.m, 6, replace=False).tolist())
        d, _ = O.check_set(prob, S)
        lo = sum(1 << j for j in S if j < 64)
        hi = sum(1 << (j - 64) for j in S if j >= 64)
        assert bool(d["optimal"]) == ((lo, hi) in listed), S
        hits += d["optimal"]
    print("level 6: optimal sets", len(opt6), "random sets found optimal", hits)


@pytest.mark.parametrize("case", list(CASES))
def test_mixed_verdicts_equal_fp64(gpu_lib, case):
    make, kmax, exh = CASES[case]
    prob = P.scale_problem(make())
    kw = dict(k_max=kmax, exhaustive=int(exh), record=1, rec_cap=4_000_000, cand_cap=1 << 20, arena_bytes=1 << 28)
    r64 = solver.solve([prob], precision=solver.FP64, **kw)
    r32 = solver.solve([prob], precision=solver.MIXED, **kw)
    assert r64.status == 0 and r32.status == 0
    a, b = _sorted(r64.rec), _sorted(r32.rec)
    assert np.array_equal(a["mask_lo"], b["mask_lo"]) and np.array_equal(a["mask_hi"], b["mask_hi"])
    for f in ("feasible", "optimal", "region"):
        bad = np.nonzero(a[f] != b[f])[0]
        assert len(bad) == 0, (f, len(bad), [(int(a["level"][i]), float(a["t"][i]), float(b["t"][i]),
                                               int(b["fp64"][i])) for i in bad[:10]])
    assert r64.total("regions") == r32.total("regions")
    print(case, "fallbacks lp1", r32.total("fallback_lp1"), "opt", r32.total("fallback_opt"), "of",
          r32.candidates, "candidates /", r32.total("feasible"), "feasible")
    # the FP64-decided values of optimal sets agree exactly
    opt = a["optimal"] == 1
    assert _same(a["t"][opt], b["t"][opt]) and _same(a["r"][opt], b["r"][opt])


def test_batch_of_instances_matches_per_instance_oracle(gpu_lib):
    probs = [P.scale_problem(p) for p in P.m62_batch(n_extra=6)]
    kmax = 2
    res = solver.solve(probs, precision=solver.FP64, k_max=kmax, record=1, rec_cap=1 << 20, cand_cap=1 << 18,
                       arena_bytes=1 << 28)
    assert res.status == 0
    for i, pr in enumerate(probs):
        ref = O.enumerate_sets(pr, k_max=kmax)
        g = _sorted(res.rec[res.rec["inst"] == i])
        o = _sorted(ref.cand)
        assert len(g) == len(o)
        for f in ("mask_lo", "mask_hi", "feasible", "optimal", "region"):
            assert np.array_equal(g[f], o[f]), (i, f)
        assert _same(g["t"], o["t"]) and _same(g["z"], o["z"])
        assert res.inst["candidates"][i] == ref.n_cand


@pytest.mark.parametrize("budget", [50, 1000, 5000])
def test_budget_truncation_matches_oracle(gpu_lib, budget):
    prob = P.scale_problem(P.random_n10_m43_p4())
    ref = O.enumerate_sets(prob, k_max=6, budget=budget, keep_records=False)
    for prec in (solver.FP64, solver.MIXED):
        res = solver.solve([prob], precision=prec, k_max=6, budget=budget, cand_cap=1 << 18, arena_bytes=1 << 28)
        assert res.status == 0
        assert res.candidates == ref.n_cand
        assert int(res.inst["truncated"][0]) == ref.truncated
        assert res.total("feasible") == ref.n_feasible
        assert res.total("regions") == ref.n_region


def _digest(sets_lo_hi):
    return sum(solver.mask_digest(lo, hi) for lo, hi in sets_lo_hi) % (1 << 64)


def test_set_digests_match_oracle(gpu_lib):
    prob = P.scale_problem(P.random_n10_m43_p4())
    ref = O.enumerate_sets(prob, k_max=3)
    for prec in (solver.FP64, solver.MIXED):
        res = solver.solve([prob], precision=prec, k_max=3, cand_cap=1 << 18, arena_bytes=1 << 28)
        c = ref.cand
        for field, dig in (("feasible", "feasible_digest"), ("optimal", "optimal_digest"),
                           ("region", "region_digest")):
            want = _digest(zip(c["mask_lo"][c[field] == 1], c["mask_hi"][c[field] == 1]))
            assert int(res.inst[dig][0]) == want, (prec, field)


def test_mixed_equals_fp64_on_the_full_bench_batch(gpu_lib):
    """Size-independent check at the bench's full size (60.8M candidates,
    33 instances): identical feasible / optimal / region sets per instance
    (order-independent 64-bit digests) and identical counts."""
    probs = [P.scale_problem(p) for p in P.m62_batch(n_extra=32)]
    kmax = [6] + [p.n for p in probs[1:]]
    budget = [0] + [1 << 19] * 32
    r32 = solver.solve(probs, precision=solver.MIXED, k_max=kmax, budget=budget, mem_fraction=0.8)
    r64 = solver.solve(probs, precision=solver.FP64, k_max=kmax, budget=budget, mem_fraction=0.8)
    assert r32.status == 0 and r64.status == 0
    for f in ("candidates", "feasible", "optimal", "regions", "feasible_digest", "optimal_digest", "region_digest",
              "truncated", "last_level"):
        assert np.array_equal(r32.inst[f], r64.inst[f]), f
    assert r32.candidates == 60802277
    # LP1 infeasible verdicts of the mixed path: the FP64 dual certificate
    # (no re-solve) or the FP64 re-solve; never more than the infeasible sets
    infeasible = r32.inst["candidates"] - r32.inst["feasible"]
    assert np.all(r32.inst["lp1_certified"] <= infeasible)
    assert r32.total("lp1_certified") > 0
    print("bench batch: infeasible", int(infeasible.sum()), "certified", r32.total("lp1_certified"),
          "cert missed", r32.total("lp1_cert_missed"), "free-variable misses", r32.total("lp1_cert_freevar"),
          "FP64 LP1 re-solves", r32.total("fallback_lp1"))


def test_mixed_equals_fp64_on_mixed_size_problems_to_full_depth(gpu_lib):
    """64 problems of mixed sizes (n <= 8, m <= 30), every active set up to
    |S| = n (3.9M candidates): the deep levels hold near-square, badly
    conditioned KKT systems, where the FP32 screen is most exposed; the
    per-instance feasible / optimal / region digests must equal FP64's, in
    both screen modes."""
    probs = [P.scale_problem(p) for p in P.pop_like_set(64, seed=0, n_max=8, m_max=30)]
    kmax = [p.n for p in probs]
    r64 = solver.solve(probs, precision=solver.FP64, k_max=kmax, mem_fraction=0.5)
    for mode in (0, 1):
        r32 = solver.solve(probs, precision=solver.MIXED, k_max=kmax, mem_fraction=0.5, lp2_screen=mode)
        assert r32.status == 0 and r64.status == 0
        for f in ("candidates", "feasible", "optimal", "regions", "feasible_digest", "optimal_digest",
                  "region_digest"):
            assert np.array_equal(r32.inst[f], r64.inst[f]), (mode, f)
    assert r64.candidates > 3_000_000


def test_mixed_equals_fp64_on_ill_conditioned_instances(gpu_lib):
    """Eight ill-conditioned instances (Q eigenvalues over four decades, 20 %
    near-duplicate rows; seeds 0..7), every set up to |S| = 4: nearly singular
    KKT systems everywhere, where an FP32 verdict is most likely to go wrong;
    the per-instance feasible / optimal / region digests must equal FP64's."""
    probs = [P.scale_problem(P.illcond_n16_m62_p8(seed=s)) for s in range(8)]
    r64 = solver.solve(probs, precision=solver.FP64, k_max=4, mem_fraction=0.5)
    r32 = solver.solve(probs, precision=solver.MIXED, k_max=4, mem_fraction=0.5)
    assert r32.status == 0 and r64.status == 0
    for f in ("candidates", "feasible", "optimal", "regions", "feasible_digest", "optimal_digest", "region_digest"):
        assert np.array_equal(r32.inst[f], r64.inst[f]), f
    print("ill-conditioned: candidates", r64.candidates, "fallbacks", r32.total("fallback_lp1"), r32.total("fallback_opt"))


def test_dual_and_primal_screens_give_the_same_verdicts(gpu_lib):
    """The FP32 optimality screen proves "not optimal" either with a dual
    bound (instances whose parameter set is a box, the default) or with the
    primal LP2 tableau; everything it cannot prove goes to the FP64 kernel.
    Both routes must end in the same feasible, optimal and region sets, with
    the same FP64 t* and r* for every optimal set.  The illcond instance has
    p = 8 and takes the primal route in both modes."""
    probs = [P.scale_problem(P.random_n10_m43_p4()), P.scale_problem(P.illcond_n16_m62_p8()),
             P.scale_problem(P.mpc_mpqp(0)), P.scale_problem(P.random_n12_m62_p6())]
    kw = dict(precision=solver.MIXED, k_max=3, record=1, rec_cap=1 << 20, cand_cap=1 << 20, arena_bytes=1 << 28)
    a = solver.solve(probs, lp2_screen=0, **kw)
    b = solver.solve(probs, lp2_screen=1, **kw)
    assert a.status == 0 and b.status == 0
    ra, rb = _sorted(a.rec, key_inst=True), _sorted(b.rec, key_inst=True)
    assert len(ra) == len(rb) == a.candidates
    for f in ("inst", "mask_lo", "mask_hi", "feasible", "optimal", "region"):
        assert np.array_equal(ra[f], rb[f]), f
    opt = ra["optimal"] == 1
    assert _same(ra["t"][opt], rb["t"][opt]) and _same(ra["r"][opt], rb["r"][opt])
    for f in ("feasible", "optimal", "regions"):
        assert a.total(f) == b.total(f), f
    # the illcond instance (p = 8) is screened the same way in both modes
    ill = ra["inst"] == 1
    assert np.array_equal(ra["lp2_status"][ill], rb["lp2_status"][ill])
    print("optimality fallbacks: dual", a.total("fallback_opt"), "primal", b.total("fallback_opt"))
