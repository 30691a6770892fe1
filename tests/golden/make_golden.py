"""Generate the golden fixtures (run here, where the reference is mounted).

    python tests/golden/make_golden.py /path/to/reference

1. ``reference_main.npz`` -- output of the reference's own Python code for a
   few seeded problems.  ``main.py`` and ``utils.py`` are imported from the
   reference checkout with three stand-ins:
     * ppopt (not installed): its constraint processing is the identity
       (no zero/duplicate/redundant rows exist in these problems);
     * gurobipy (not installed): a minimal Model backed by scipy HiGHS that
       records every Chebyshev radius it solves (utils.py:72-86);
     * the ctypes library ``mpqp_cuda.so`` (missing from the reference): a
       fake whose ``mpqp`` records the LP matrices main.py builds
       (main.py:87-144) and answers with the optimal active sets of the C
       oracle, so that main.py continues into active_sets_to_regions
       (utils.py:100-144) exactly as written.
   Stored per problem: the raw data, the LP matrices captured at the ctypes
   boundary, the scaled problem utils.py computes regions on, and every
   region dict plus its radius.
2. ``exact_verdicts.json`` -- exact rational feasibility / optimality
   verdicts (oracle/exact_lp.py) of every active set with |S| <= n of the
   small problems, the known answers the oracle is pinned to.
"""
from __future__ import annotations

import ctypes
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mpqpcudasolver_gb300 import problems as P  # noqa: E402
from oracle import exact_lp as X  # noqa: E402
from oracle import oracle as O  # noqa: E402

# problems of the fixtures: (label, generator)
PROBLEMS = [
    ("n4m10p2", lambda: P.random_n4_m10_p2()),
    ("rand-n3-m8-p2-s11", lambda: P.random_mpqp(3, 8, 2, seed=11)),
    ("rand-n4-m12-p3-s12", lambda: P.random_mpqp(4, 12, 3, seed=12)),
    ("rand-n5-m14-p2-s13", lambda: P.random_mpqp(5, 14, 2, seed=13)),
    ("mpc-h2-s0", lambda: P.mpc_mpqp(0, horizon=2)),
]


def _install_stubs(radii: list):
    from scipy.optimize import linprog

    # ppopt: identity constraint processing
    ppopt = types.ModuleType("ppopt")
    utils_m = types.ModuleType("ppopt.utils")
    cu = types.ModuleType("ppopt.utils.constraint_utilities")
    cu.process_program_constraints = lambda A, b, F, A_t, b_t: (A, b, F, A_t, b_t)
    cu.find_implicit_equalities = lambda A, b, F, eq: (A, b, F, eq)
    cu.find_redundant_constraints = lambda A, b, eq, solver=None: list(range(A.shape[0]))
    gu = types.ModuleType("ppopt.utils.general_utils")
    gu.ppopt_block = np.block
    sol = types.ModuleType("ppopt.solver")

    class Solver:
        def __init__(self):
            self.solvers = {"lp": None}
    sol.Solver = Solver
    prog = types.ModuleType("ppopt.mpqp_program")
    prog.MPQP_Program = object
    mps = types.ModuleType("ppopt.mp_solvers")
    smq = types.ModuleType("ppopt.mp_solvers.solve_mpqp")
    smq.solve_mpqp = None
    smq.mpqp_algorithm = types.SimpleNamespace(combinatorial=0, combinatorial_parallel=1)
    for name, mod in [("ppopt", ppopt), ("ppopt.utils", utils_m), ("ppopt.utils.constraint_utilities", cu),
                      ("ppopt.utils.general_utils", gu), ("ppopt.solver", sol), ("ppopt.mpqp_program", prog),
                      ("ppopt.mp_solvers", mps), ("ppopt.mp_solvers.solve_mpqp", smq)]:
        sys.modules[name] = mod

    # gurobipy: the subset utils.py uses, solved with HiGHS
    gp = types.ModuleType("gurobipy")

    class GRB:
        INFINITY = float("inf")
        MAXIMIZE = -1
        OPTIMAL = 2
        SUBOPTIMAL = 13
        INFEASIBLE = 3

    class MVar:
        def __init__(self, n):
            self.n = n
            self.X = np.full(n, np.nan)

        def __getitem__(self, i):
            return ("var", i % self.n)

    class Model:
        def __init__(self):
            self.x = None
            self.A = None
            self.b = None
            self.obj = None
            self.status = None

        def setParam(self, *a):
            pass

        def addMVar(self, n, lb=None, ub=None):
            self.x = MVar(n)
            return self.x

        def addMConstr(self, A, x, sense, b):
            assert sense == "<"
            self.A, self.b = np.asarray(A, float), np.asarray(b, float)

        def setObjective(self, expr, sense=None):
            self.obj = (expr[1], sense)

        def optimize(self):
            n = self.x.n
            cost = np.zeros(n)
            cost[self.obj[0]] = -1.0 if self.obj[1] == GRB.MAXIMIZE else 1.0
            res = linprog(cost, A_ub=self.A, b_ub=self.b, bounds=(None, None), method="highs")
            if res.status == 0:
                self.status = GRB.OPTIMAL
                self.x.X = res.x
                radii.append(float(res.x[-1]))
            else:
                self.status = GRB.INFEASIBLE
                radii.append(float("nan"))

        def update(self):
            pass

    gp.Model = Model
    gp.GRB = GRB
    sys.modules["gurobipy"] = gp
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt


class _FakeLib:
    """Stands in for mpqp_cuda.so: records the call, answers with the oracle."""

    def __init__(self, gpu_results_cls):
        self.cls = gpu_results_cls
        self.calls = []
        self.keep = []
        self.mpqp = self._mpqp
        self.warm_up = lambda: None

    def _mpqp(self, A0, n_c, n_x, n_t, k_min, k_max, extra, A1, xb1, b1, M1, N1, A2, xb2, b2, non_b2, M2, N2,
              n_eqs, reserved):
        def arr(ptr, shape, dtype=np.float64, order="F"):
            n = int(np.prod(shape))
            a = np.ctypeslib.as_array(ptr, shape=(n,)).copy()
            return a.reshape(shape, order=order).astype(dtype)
        cap = dict(A0=arr(A0, (n_x, n_c)), A1=arr(A1, (M1, N1)), xb1=arr(xb1, (M1,), order="C"),
                   b1=arr(b1, (M1,), np.intc, "C"), A2=arr(A2, (M2, N2)), xb2=arr(xb2, (M2,), order="C"),
                   b2=arr(b2, (M2,), np.intc, "C"), non_b2=arr(non_b2, (N2 - M2,), np.intc, "C"),
                   dims=np.array([n_c, n_x, n_t, k_min, k_max, extra, M1, N1, M2, N2, n_eqs, reserved]))
        # the problem main.py passed, read back from its LP1 / LP2 blocks
        n_cp = M1 - n_c
        A = cap["A1"][:n_c, :n_x]
        F = -cap["A1"][:n_c, n_x:n_x + n_t]
        At = cap["A1"][n_c:, n_x:n_x + n_t]
        r0 = n_c + 1 + n_cp
        s = np.sign(np.diag(cap["A2"][r0:r0 + n_x, :n_x]))
        Q = s[:, None] * cap["A2"][r0:r0 + n_x, :n_x]
        H = s[:, None] * cap["A2"][r0:r0 + n_x, n_x:n_x + n_t]
        c = -s * cap["xb2"][r0:r0 + n_x]
        prob = P.MPQP(Q, c, H, A, cap["xb1"][:n_c].copy(), F, At, cap["xb1"][n_c:].copy())
        e = O.enumerate_sets(prob, k_min=k_min, k_max=k_max)
        opt = [O.mask_to_set(r["mask_lo"], r["mask_hi"]) for r in e.cand if r["optimal"]]
        cap["oracle_counts"] = np.array([e.n_cand, e.n_feasible, e.n_optimal, e.n_region])
        rows = np.full((max(len(opt), 1), n_x), -1, dtype=np.intc)
        for i, S in enumerate(opt):
            rows[i, :len(S)] = S
        self.calls.append(cap)
        res = self.cls()
        res.n_batches = 1
        res.n_splits = 1
        res.n_feasible_lps = e.n_feasible
        res.n_final_lps = len(opt)
        res.time_feas = res.time_opti = res.time_GPU = 0.0
        buf = np.ascontiguousarray(rows.ravel())
        self.keep.append(buf)
        res.active_sets = buf.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        self.keep.append(res)
        return ctypes.pointer(res)


def make_reference_fixtures(ref_dir: str) -> dict:
    radii: list = []
    _install_stubs(radii)
    sys.path.insert(0, ref_dir)
    import main as ref_main  # the reference's driver
    import utils as ref_utils  # noqa: F401  the reference's region code

    captured = {}
    real_loader = ctypes.cdll.LoadLibrary
    fakes = []

    def fake_loader(name):
        # GPUResults is defined inside calculate_mpqp_with_CUDA; take the
        # restype class main.py assigns (main.py:50) when it does so
        class Hook(_FakeLib):
            def __setattr__(self, k, v):
                object.__setattr__(self, k, v)
        h = Hook(None)

        class M:
            def __init__(self, outer):
                self.outer = outer
                self.argtypes = None
                self._restype = None

            @property
            def restype(self):
                return self._restype

            @restype.setter
            def restype(self, v):
                self._restype = v
                self.outer.cls = v._type_

            def __call__(self, *a):
                return self.outer._mpqp(*a)
        h.mpqp = M(h)
        fakes.append(h)
        return h

    ctypes.cdll.LoadLibrary = fake_loader
    try:
        for label, gen in PROBLEMS:
            prob = gen()
            data = {"A": prob.A, "b": prob.b.reshape(-1, 1), "c": prob.c.reshape(-1, 1), "F": prob.F,
                    "Q": prob.Q, "CRA": prob.CRA, "CRb": prob.CRb.reshape(-1, 1), "Ht": prob.H}
            radii.clear()
            regions_seen = []
            orig = ref_main.active_sets_to_regions

            def spy(prog, sets, _orig=orig):
                sol = _orig(prog, sets)
                regions_seen.append((prog, sol))
                return sol
            ref_main.active_sets_to_regions = spy
            out = ref_main.calculate_mpqp_with_CUDA([data], [0])
            ref_main.active_sets_to_regions = orig
            cap = fakes[-1].calls[-1]
            prog, sol = regions_seen[-1]
            entry = {f"{label}/raw/{k}": np.asarray(v) for k, v in data.items()}
            for k, v in cap.items():
                entry[f"{label}/lp/{k}"] = v
            # problem utils.py computed the regions on (scale_method=2)
            for k, v in (("A", prog.A), ("b", prog.b), ("c", prog.c), ("F", prog.F), ("Q", prog.Q),
                         ("H", prog.H), ("CRA", prog.A_t), ("CRb", prog.b_t)):
                entry[f"{label}/prog/{k}"] = np.asarray(v, dtype=np.float64)
            entry[f"{label}/n_regions"] = np.array([len(sol), int(out[0, 1])])
            entry[f"{label}/radii"] = np.array(radii, dtype=np.float64)
            for i, reg in enumerate(sol):
                for k in ("parameter_A", "parameter_b", "lagrange_A", "lagrange_b", "CR_As", "CR_bs"):
                    entry[f"{label}/region{i}/{k}"] = np.asarray(reg[k], dtype=np.float64)
                entry[f"{label}/region{i}/active_set"] = np.asarray(reg["active_set"], dtype=np.int64)
            captured.update(entry)
            print(f"{label}: {len(sol)} regions, {len(radii)} Chebyshev LPs, oracle counts {cap['oracle_counts']}")
    finally:
        ctypes.cdll.LoadLibrary = real_loader
    return captured


def make_exact_fixtures() -> dict:
    out = {}
    for label, gen in PROBLEMS[:4]:
        prob = P.scale_problem(gen())
        v = X.exhaustive_verdicts(prob, prob.n)
        out[label] = {"k_max": prob.n,
                      "feasible": [list(S) for S, d in v.items() if d["feasible"]],
                      "optimal": [list(S) for S, d in v.items() if d["optimal"]],
                      "n_sets": len(v)}
        print(f"{label}: exact {len(v)} sets, {len(out[label]['feasible'])} feasible, "
              f"{len(out[label]['optimal'])} optimal")
    return out


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else None
    ex = make_exact_fixtures()
    with open(os.path.join(HERE, "exact_verdicts.json"), "w") as f:
        json.dump(ex, f, indent=0)
    if ref:
        fx = make_reference_fixtures(ref)
        np.savez_compressed(os.path.join(HERE, "reference_main.npz"), **fx)
