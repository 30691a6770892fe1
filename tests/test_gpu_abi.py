"""The drop-in boundary on the GPU: mpqp() called through ctypes exactly as
the reference's main.py calls mpqp_cuda.so (main.py:25-50,60,144), and the
host mirror of main.py's loop, against the oracle and the reference's own
regions (golden fixtures)."""
import os

import numpy as np
import pytest

from mpqpcudasolver_gb300 import host
from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GEN = {
    "n4m10p2": lambda: P.random_n4_m10_p2(),
    "rand-n3-m8-p2-s11": lambda: P.random_mpqp(3, 8, 2, seed=11),
    "rand-n4-m12-p3-s12": lambda: P.random_mpqp(4, 12, 3, seed=12),
    "rand-n5-m14-p2-s13": lambda: P.random_mpqp(5, 14, 2, seed=13),
    "mpc-h2-s0": lambda: P.mpc_mpqp(0, horizon=2),
}


@pytest.fixture(scope="module")
def ref():
    return dict(np.load(os.path.join(GOLDEN, "reference_main.npz")))


@pytest.mark.parametrize("label", list(GEN))
@pytest.mark.parametrize("precision", ["default", "fp64", "mixed"])
def test_mpqp_drop_in_matches_oracle_and_reference(gpu_lib, ref, label, precision, monkeypatch):
    """No environment variable: mpqp() runs in mixed precision, the same sets
    as the FP64 kernels and the oracle."""
    if precision == "default":
        monkeypatch.delenv("MPQP_PRECISION", raising=False)
    else:
        monkeypatch.setenv("MPQP_PRECISION", precision)
    lib = host.load_mpqp_cuda()
    lib.warm_up()
    prog = host.MPQPProb.from_mpqp(GEN[label]())
    prog.process_constraints(scale_method=1)
    d = host.build_lp_data(prog)
    r = host.call_mpqp(lib, d)
    g = r.contents
    assert g.status == 0, solver.last_error()
    e = O.enumerate_sets(prog.to_mpqp(), k_max=d["num_x"])
    sets = host.decode_active_sets(g.active_sets, g.n_final_lps, d["num_x"])
    want = sorted(O.mask_to_set(c["mask_lo"], c["mask_hi"]) for c in e.cand if c["optimal"])
    assert sorted(sets) == want
    assert g.n_feasible_lps == e.n_feasible and g.n_candidates == e.n_cand
    assert g.n_regions == e.n_region == int(ref[f"{label}/n_regions"][0])
    assert g.time_GPU > 0 and g.n_batches >= 1
    # the device time split like main.py:18-20 reads it
    assert g.time_feas > 0 and g.time_opti > 0
    assert g.time_feas + g.time_opti <= g.time_GPU * 1.001 + 1e-6
    lib.mpqp_free(r)


def test_mpqp_reports_malformed_layout_without_gpu_work(gpu_lib):
    lib = host.load_mpqp_cuda()
    prog = host.MPQPProb.from_mpqp(P.random_n4_m10_p2())
    prog.process_constraints(scale_method=1)
    d = host.build_lp_data(prog)
    d = dict(d, M2=d["M2"] - 1)
    r = host.call_mpqp(lib, d)
    assert r.contents.status == solver.ELAYOUT and r.contents.n_final_lps == 0
    lib.mpqp_free(r)


def test_k_min_filters_reported_sets(gpu_lib):
    lib = host.load_mpqp_cuda()
    prog = host.MPQPProb.from_mpqp(P.random_mpqp(4, 12, 3, seed=12))
    prog.process_constraints(scale_method=1)
    d = host.build_lp_data(prog)
    r = host.call_mpqp(lib, d, k_min=2).contents
    sets = host.decode_active_sets(r.active_sets, r.n_final_lps, d["num_x"])
    e = O.enumerate_sets(prog.to_mpqp(), k_min=2, k_max=d["num_x"])
    want = sorted(O.mask_to_set(c["mask_lo"], c["mask_hi"]) for c in e.cand if c["optimal"] and c["level"] >= 2)
    assert sorted(sets) == want and all(len(s) >= 2 for s in sets)


def test_calculate_mpqp_with_cuda_region_counts_match_reference(gpu_lib, ref):
    probs = [GEN[k]() for k in GEN]
    rows, raw = host.calculate_mpqp_with_CUDA(probs)
    for i, label in enumerate(GEN):
        assert int(rows[i, 1]) == int(ref[f"{label}/n_regions"][0]), label


@pytest.mark.parametrize("label", list(GEN))
def test_regions_pass_enumerates_nothing(gpu_lib, ref, label, monkeypatch):
    """main.py:144-157: mpqp() returns the optimal sets, then the regions pass
    forms each region (utils.py:128-144).  Both ways of the pass -- with the
    radius test mpqp() already ran (GPUResults.is_region) and with the radii
    computed beside the laws -- keep the reference's regions and launch no
    enumeration (solver.solve is not called)."""
    lib = host.load_mpqp_cuda()
    prog = host.MPQPProb.from_mpqp(GEN[label]())
    prog.process_constraints(scale_method=1)
    d = host.build_lp_data(prog)
    r = host.call_mpqp(lib, d)
    g = r.contents
    assert g.status == 0
    prog.num_x = d["num_x"]
    prog.n_active_sets = g.n_final_lps

    def no_enumeration(*a, **k):
        raise AssertionError("the regions pass enumerated")
    monkeypatch.setattr(solver, "solve", no_enumeration)
    a = host.active_sets_to_regions(prog, g.active_sets, g.is_region)
    b = host.active_sets_to_regions(prog, g.active_sets)
    want = int(ref[f"{label}/n_regions"][0])
    assert len(a) == len(b) == g.n_regions == want
    for x, y in zip(a, b):
        assert x["active_set"] == y["active_set"]
        assert np.array_equal(x["parameter_A"], y["parameter_A"])
    radii = sorted(y["r"] for y in b)
    assert all(rr >= 1e-8 for rr in radii)
    lib.mpqp_free(r)


@pytest.mark.parametrize("label", list(GEN))
def test_device_region_laws_match_reference_regions(gpu_lib, ref, label):
    pk = {k: ref[f"{label}/prog/{k}"] for k in ("A", "b", "c", "F", "Q", "H", "CRA", "CRb")}
    prob = P.MPQP(pk["Q"], pk["c"].ravel(), pk["H"], pk["A"], pk["b"].ravel(), pk["F"], pk["CRA"], pk["CRb"].ravel())
    sets, i = [], 0
    while f"{label}/region{i}/active_set" in ref:
        sets.append([int(s) for s in ref[f"{label}/region{i}/active_set"]])
        i += 1
    laws = solver.region_laws(prob, sets)
    for i, law in enumerate(laws):
        for key in ("lagrange_A", "parameter_A", "lagrange_b", "parameter_b"):
            b = ref[f"{label}/region{i}/{key}"].reshape(law[key].shape)
            assert np.allclose(law[key], b, rtol=1e-8, atol=1e-12), (i, key)
        As, bs = ref[f"{label}/region{i}/CR_As"], ref[f"{label}/region{i}/CR_bs"].ravel()
        keep = np.abs(bs) < 1e10
        assert np.allclose(law["CR_As"], As[keep], rtol=1e-8, atol=1e-12)
        assert np.allclose(law["CR_bs"], bs[keep], rtol=1e-8, atol=1e-12)
    res = solver.solve([prob], precision=solver.FP64, k_max=prob.n, cand_cap=1 << 16, arena_bytes=1 << 26)
    radii = {tuple(solver.mask_to_set(o["mask_lo"], o["mask_hi"])): o["r"] for o in res.opt if o["region"]}
    for i, S in enumerate(sets):
        r_ref = ref[f"{label}/radii"][i]
        assert abs(radii[tuple(S)] - r_ref) <= 1e-8 * max(1.0, abs(r_ref))
