"""Run one enumeration of a named workload, for profilers and quick timing.

    python -m mpqpcudasolver_gb300.profile_case CASE [--precision mixed|fp64] [--runs R]

CASE: m62-k3 | m62-k4 | m62-k5 (the n=12, m=62, p=6 instance up to |S| = k)
| m62-batch (the bench batch) | n10m43p4-k4 | illcond-k3 | mpc-batch (64 MPC
instances, |S| <= 3) | pop-like (64 problems of mixed sizes, n <= 8, m <= 30,
every |S| <= n) | mplp-batch (32 mpLPs, Q = 0, every |S| <= n).
Prints one JSON line with the candidates, the device time of the last run
and the per-kernel times of a timed run.
"""
from __future__ import annotations

import argparse
import json
import sys

from . import problems as P
from . import solver


def workload(case: str):
    if case.startswith("m62-k"):
        return [P.scale_problem(P.random_n12_m62_p6())], int(case.rsplit("k", 1)[1]), 0
    if case == "m62-batch":
        probs = [P.scale_problem(p) for p in P.m62_batch(n_extra=32)]
        return probs, [6] + [p.n for p in probs[1:]], [0] + [1 << 19] * 32
    if case == "n10m43p4-k4":
        return [P.scale_problem(P.random_n10_m43_p4())], 4, 0
    if case == "illcond-k3":
        return [P.scale_problem(P.illcond_n16_m62_p8())], 3, 0
    if case == "pop-like":
        probs = [P.scale_problem(p) for p in P.pop_like_set(64, seed=0, n_max=8, m_max=30)]
        return probs, [p.n for p in probs], 0
    if case == "mplp-batch":
        probs = [P.scale_problem(p) for p in P.mplp_batch()]
        return probs, [p.n for p in probs], 0
    if case == "mpc-batch":
        return [P.scale_problem(p) for p in P.mpc_batch(64)], 3, 0
    raise SystemExit(f"unknown case {case}")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--runs", type=int, default=1)
    ap.add_argument("--mem-fraction", type=float, default=0.85,
                    help="share of free device memory the plan may take (arenas are also capped by the "
                         "combinatorial size of the workload)")
    ap.add_argument("--lp2-screen", type=int, default=0,
                    help="FP32 optimality screen: 0 dual bound on box instances, 1 primal tableau screen")
    args = ap.parse_args(argv)
    probs, kmax, budget = workload(args.case)
    prec = solver.MIXED if args.precision == "mixed" else solver.FP64
    extra = {"lp2_screen": args.lp2_screen}
    plan = solver.Plan(probs, precision=prec, k_max=kmax, budget=budget, mem_fraction=args.mem_fraction, **extra)
    for _ in range(args.runs):
        plan.run()
    r = plan.results()
    plan.run_timed()
    kt = plan.kernel_times()
    r2 = plan.results()
    print(json.dumps({"case": args.case, "precision": args.precision, "candidates": r.candidates,
                      "feasible": r.total("feasible"), "optimal": r.total("optimal"), "regions": r.total("regions"),
                      "device_ms": r.device_ms, "timed_ms": r2.device_ms,
                      "cand_per_s": r.candidates / (r.device_ms / 1e3),
                      "kernels": {k: [round(v[0], 3), v[1]] for k, v in kt.items()},
                      "fallbacks": [r.total("fallback_lp1"), r.total("fallback_opt")],
                      "lp2_certified": r.total("lp2_certified")}))
    plan.close()
    if r.status != 0 or r2.status != 0:
        print(f"status {r.status} / {r2.status}: {solver.last_error()}", file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
