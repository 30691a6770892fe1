"""Run one enumeration of a named workload, for profilers and quick timing.

    python -m mpqpcudasolver_gb300.profile_case CASE [--precision mixed|fp64] [--runs R]

CASE: config3main-k3 | config3main-k4 | config3main-k5 | config3 (the bench
batch) | config2-k4 | config4-k3 | config5 (64 MPC instances, |S| <= 3).
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
    if case.startswith("config3main-k"):
        return [P.scale_problem(P.config3_main())], int(case.rsplit("k", 1)[1]), 0
    if case == "config3":
        probs = [P.scale_problem(p) for p in P.config3(n_extra=32)]
        return probs, [6] + [p.n for p in probs[1:]], [0] + [1 << 19] * 32
    if case == "config2-k4":
        return [P.scale_problem(P.config2())], 4, 0
    if case == "config4-k3":
        return [P.scale_problem(P.config4())], 3, 0
    if case == "config5":
        return [P.scale_problem(p) for p in P.config5(64)], 3, 0
    raise SystemExit(f"unknown case {case}")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--runs", type=int, default=1)
    args = ap.parse_args(argv)
    probs, kmax, budget = workload(args.case)
    prec = solver.MIXED if args.precision == "mixed" else solver.FP64
    plan = solver.Plan(probs, precision=prec, k_max=kmax, budget=budget, mem_fraction=0.85)
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
                      "fallbacks": [r.total("fallback_lp1"), r.total("fallback_opt")]}))
    plan.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
