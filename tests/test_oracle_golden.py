"""The oracle pinned to known answers and to the reference's own code (CPU).

* exact_verdicts.json: exact rational verdicts of every active set with
  |S| <= n of four small problems (oracle/exact_lp.py).
* reference_main.npz: what the reference's main.py / utils.py produced for
  five problems (tests/golden/make_golden.py): the LP matrices at the ctypes
  boundary and every critical region with its Chebyshev radius.
"""
import json
import os

import numpy as np
import pytest

from mpqpcudasolver_gb300 import host
from mpqpcudasolver_gb300 import problems as P
from oracle import oracle as O
from oracle import reference_lp as R

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GEN = {
    "n4m10p2": lambda: P.random_n4_m10_p2(),
    "rand-n3-m8-p2-s11": lambda: P.random_mpqp(3, 8, 2, seed=11),
    "rand-n4-m12-p3-s12": lambda: P.random_mpqp(4, 12, 3, seed=12),
    "rand-n5-m14-p2-s13": lambda: P.random_mpqp(5, 14, 2, seed=13),
    "mpc-h2-s0": lambda: P.mpc_mpqp(0, horizon=2),
}


@pytest.fixture(scope="module")
def exact():
    with open(os.path.join(GOLDEN, "exact_verdicts.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def ref():
    return dict(np.load(os.path.join(GOLDEN, "reference_main.npz")))


def _sets(cand, field):
    return sorted(tuple(O.mask_to_set(c["mask_lo"], c["mask_hi"])) for c in cand if c[field])


@pytest.mark.parametrize("label", ["n4m10p2", "rand-n3-m8-p2-s11", "rand-n4-m12-p3-s12", "rand-n5-m14-p2-s13"])
def test_oracle_matches_exact_rational_verdicts(exact, label):
    fx = exact[label]
    prob = P.scale_problem(GEN[label]())
    e = O.enumerate_sets(prob, k_max=fx["k_max"], exhaustive=True)
    assert e.n_cand == fx["n_sets"]
    assert _sets(e.cand, "feasible") == sorted(tuple(s) for s in fx["feasible"])
    assert _sets(e.cand, "optimal") == sorted(tuple(s) for s in fx["optimal"])
    # with pruning the same sets are found (infeasibility is inherited by supersets)
    ep = O.enumerate_sets(prob, k_max=fx["k_max"])
    assert _sets(ep.cand, "feasible") == sorted(tuple(s) for s in fx["feasible"])
    assert _sets(ep.cand, "optimal") == sorted(tuple(s) for s in fx["optimal"])


@pytest.mark.parametrize("label", list(GEN))
def test_lp_matrices_match_reference_main(ref, label):
    """host.build_lp_data restates main.py:87-137; the reference's own code built these."""
    raw = GEN[label]()
    prog = host.MPQPProb.from_mpqp(raw)
    prog.process_constraints(scale_method=1)
    d = host.build_lp_data(prog)
    for k in ("A0", "A1", "A2"):
        assert np.array_equal(d[k], ref[f"{label}/lp/{k}"]), k
    for k in ("xb1", "xb2"):
        assert np.array_equal(d[k].ravel(), ref[f"{label}/lp/{k}"]), k
    for k in ("b1", "b2", "non_b2"):
        assert np.array_equal(d[k], ref[f"{label}/lp/{k}"]), k
    dims = ref[f"{label}/lp/dims"]
    assert (d["num_c"], d["num_x"], d["num_t"]) == tuple(dims[:3])
    assert (d["M1"], d["N1"], d["M2"], d["N2"], d["n_eqs"]) == tuple(dims[6:11])


@pytest.mark.parametrize("label", list(GEN))
def test_regions_match_reference_utils(ref, label):
    """Laws, normalised region rows and radii of every region the reference's
    utils.py formed (on its scale_method=2 problem) -- within 1e-8 relative."""
    pk = {k: ref[f"{label}/prog/{k}"] for k in ("A", "b", "c", "F", "Q", "H", "CRA", "CRb")}
    prob = P.MPQP(pk["Q"], pk["c"].ravel(), pk["H"], pk["A"], pk["b"].ravel(), pk["F"], pk["CRA"], pk["CRb"].ravel())
    n_reg = int(ref[f"{label}/n_regions"][0])
    radii = ref[f"{label}/radii"]
    assert n_reg > 0
    i = 0
    while f"{label}/region{i}/active_set" in ref:
        S = [int(s) for s in ref[f"{label}/region{i}/active_set"]]
        rec, law = O.check_set(prob, S, want_laws=True)
        assert rec["region"] == 1, S
        # 1e-8 relative per entry, 1e-12 absolute floor (entries that are zero
        # in exact arithmetic carry only rounding noise on both sides)
        for key in ("lagrange_A", "parameter_A", "lagrange_b", "parameter_b"):
            b = ref[f"{label}/region{i}/{key}"].reshape(law[key].shape)
            assert np.allclose(law[key], b, rtol=1e-8, atol=1e-12), (S, key)
        # normalised rows: the reference keeps rows that are zero up to
        # rounding (they normalise to |CR_bs| ~ 1e15); drop those before comparing
        As, bs = ref[f"{label}/region{i}/CR_As"], ref[f"{label}/region{i}/CR_bs"].ravel()
        keep = np.abs(bs) < 1e10
        assert law["CR_As"].shape == As[keep].shape, S
        assert np.allclose(law["CR_As"], As[keep], rtol=1e-8, atol=1e-12), S
        assert np.allclose(law["CR_bs"], bs[keep], rtol=1e-8, atol=1e-12), S
        assert abs(rec["r"] - radii[i]) <= 1e-8 * max(1.0, abs(radii[i])), (S, rec["r"], radii[i])
        i += 1
    assert i == n_reg


@pytest.mark.parametrize("label", list(GEN))
def test_verdicts_match_reference_lps_solved_by_highs(ref, label):
    """Every candidate's LP1 / LP2 verdict equals HiGHS on the LP matrices the
    reference's main.py built (specialised per set as batched_simplex.cu does)."""
    mats = {k: ref[f"{label}/lp/{k}"] for k in ("A1", "A2", "b1", "b2", "non_b2")}
    mats["xb1"] = ref[f"{label}/lp/xb1"].reshape(-1, 1)
    mats["xb2"] = ref[f"{label}/lp/xb2"].reshape(-1, 1)
    dims = ref[f"{label}/lp/dims"]
    n_c, n_x, n_t = (int(v) for v in dims[:3])
    mats.update(M1=int(dims[6]), N1=int(dims[7]), M2=int(dims[8]), N2=int(dims[9]), n_eqs=int(dims[10]), n_c=n_c,
                n_x=n_x, n_t=n_t)
    prob = P.scale_problem(GEN[label]())
    e = O.enumerate_sets(prob)
    rng = np.random.default_rng(0)
    idx = np.arange(len(e.cand))
    if len(idx) > 400:
        idx = np.unique(np.concatenate([rng.choice(idx, 300, replace=False), np.nonzero(e.cand["optimal"])[0],
                                        np.nonzero(e.cand["feasible"] == 0)[0][:100]]))
    for i in idx:
        c = e.cand[i]
        S = O.mask_to_set(c["mask_lo"], c["mask_hi"])
        z = R.lp1_value(mats, S)
        assert (z <= 1e-9) == bool(c["feasible"]), (S, z, c["z"])
        if c["feasible"] and c["licq"]:
            t = R.lp2_value(mats, S)
            assert (t > 1e-9) == bool(c["optimal"]), (S, t, c["t"])
    assert e.n_region == int(ref[f"{label}/n_regions"][0])
