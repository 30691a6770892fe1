#!/usr/bin/env python
"""Benchmark: candidate active sets checked per second at m = 62.

Workload (one "step" = one full enumeration of it, all levels, one launch
sequence): the m = 62 batch -- a random mpQP with n=12, m=62, p=6 whose
candidate active sets of cardinality 0..6 are all checked (54.3M candidates),
plus 32 random instances (seeds 1..32, n~U{5..15}, m~U{20..80}, p~U{2..6})
enumerated up to |S| = n under a budget of 2^19 candidates each.  Inputs are
seeded synthetic problems (no dataset exists for this metric).

Our arm (default): the mixed-precision path (FP32 pivots and KKT solves, FP64
certificates / re-solves) on a device-resident plan; the plain FP64 path runs
once on the same workload for the speed-up and the identical-regions check.
`--impl reference` times the CPU restatement of the reference's algorithm
(the C oracle, all host threads) on a bounded sample of the same workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "candidate active sets checked/s at m=62 (mixed FP32/FP64 vs FP64), same regions"
UNIT = "candidates/s"
EXTRA_BUDGET = 1 << 19
MAIN_KMAX = 6
# CPU sample of the same workload: the main instance's active sets drawn only
# from its last 40 constraints (a family closed under subsets, so all six
# levels with the full enumeration's subset tests, warm starts and LPs), plus
# 3 of the 32 extra instances at their full budget
CPU_TAIL_FIRST = 22
CPU_EXTRAS = 3
# single-core figure: the last 28 constraints only
CPU_TAIL_FIRST_1CORE = 34
DETAIL_FILE = "bench_detail.json"


def workload():
    from mpqpcudasolver_gb300 import problems as P
    probs = [P.scale_problem(p) for p in P.m62_batch(n_extra=32)]
    kmax = [MAIN_KMAX] + [p.n for p in probs[1:]]
    budget = [0] + [EXTRA_BUDGET] * (len(probs) - 1)
    return probs, kmax, budget


def config_dict(precision: str) -> dict:
    return {"workload": f"m62 batch: random mpQP n=12 m=62 p=6, all active sets |S|<=6, plus 32 random mpQPs "
                        f"(seeds 1..32, n~U{{5..15}}, m~U{{20..80}}, p~U{{2..6}}) up to |S|=n, budget "
                        f"{EXTRA_BUDGET} candidates each; one launch sequence per step",
            "precision": precision, "instances": 33, "m": 62, "n": 12, "p": 6,
            "l2": "flushed between steps (512 MiB write); working set (LP1 tableaus) also exceeds L2"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [x.strip() for x in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())
                if any(r[3].replace(".", "").isdigit() for r in rows) else None}


def measured_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "source": "fallback"}


def lp1_unique_bytes(res) -> float:
    """Algorithmic bytes of all LP1 (k_feasibility) launches of one step,
    each item counted once (device counters of the run):

    * every distinct parent whose children were checked: its live tableau
      rows and objective row, basis ids and 48 B node (read once; its other
      children find it in L2);
    * per checked candidate (levels >= 1): the 8 B candidate record (read) and
      its 48 B node slot (written);
    * per stored child: its live tableau rows, ids (write) and its 8 B hash
      slot; per certificate-queue entry 32 B, per FP64 re-solve entry 4 B.

    Last-level children decided at a certified vertex do not load their
    parent, so when all children of a parent are decided that way the model
    charges a tableau that is not read."""
    total = 0.0
    for st in res.inst:
        cand = int(st["candidates"]) - 1          # level 0 (the empty set) is set up by k_level0
        total += int(st["lp1_parent_bytes"]) + int(st["lp1_store_bytes"]) + cand * (8 + 48)
        total += int(st["stored"]) * 8 + (int(st["lp1_certified"]) + int(st["lp1_cert_missed"])) * 32
        total += int(st["fallback_lp1"]) * 4
    return float(total)


def profile_figure(name: str, key: str):
    """A per-unit figure recorded from an ncu capture under profiles/."""
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            return float(json.load(f)[key])
    except Exception:
        return None


def opt_algorithmic_bytes(probs, res, elem: int) -> float:
    """Algorithmic bytes of all optimality (k_optimality) launches of one step.

    Per evaluated set (every feasible set, the empty set included): the
    shared-data gather for the KKT rows 8*m*(n+p+1), the region tableau
    written once 8*R*(p+2) (R = m + rows of the parameter box) and the 16 B
    mask and verdict; per LP2 / Chebyshev pivot one read and one write of the
    (R+1) x (p+2) tableau at the pivot element size.
    """
    total = 0.0
    for i, pr in enumerate(probs):
        st = res.inst[i]
        m, n, p = pr.m, pr.n, pr.p
        R = m + pr.CRA.shape[0]
        total += int(st["feasible"]) * (8 * m * (n + p + 1) + 8 * R * (p + 2) + 16)
        total += 2 * elem * (int(st["lp2_pivots"]) + int(st["cheb_pivots"])) * (R + 1) * (p + 2)
    return float(total)


def traffic_per_launch(name: str, units_per_launch: float):
    """DRAM bytes per launch, scaled from an ncu capture of a smaller case
    (bytes per unit, recorded under profiles/) to this launch's units."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            per_unit = float(json.load(f)["dram_bytes_per_unit"])
    except Exception:
        return None
    return per_unit * units_per_launch


def model_bytes_touched(probs, res, elem: int) -> float:
    """Bytes-touched model of the hot path (scratchpad + HBM), per step:
    8*m*(n+p+1) shared-data gather + 8*R*(p+2) region tableau per evaluated
    set, plus 2*R_LP*C_LP*s per pivot, plus 16 B mask and verdict."""
    total = 0.0
    for i, pr in enumerate(probs):
        st = res.inst[i]
        m, n, p = pr.m, pr.n, pr.p
        R = m + pr.CRA.shape[0]
        lp1 = (R + 1) * (n + p + 1)
        lp2 = (R + 1) * (p + 2)
        total += st["candidates"] * 16 + st["feasible"] * (8 * m * (n + p + 1) + 8 * R * (p + 2))
        total += 2 * elem * (st["lp1_pivots"] * lp1 + (st["lp2_pivots"] + st["cheb_pivots"]) * lp2)
    return float(total)


def same_regions(a, b) -> bool:
    ka = {(int(o["inst"]), int(o["mask_lo"]), int(o["mask_hi"])) for o in a.opt if o["region"]}
    kb = {(int(o["inst"]), int(o["mask_lo"]), int(o["mask_hi"])) for o in b.opt if o["region"]}
    return ka == kb and len(a.opt) == len(b.opt)


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        import torch
        torch.cuda.set_device(local)
        dist_mod.init_process_group(backend="nccl")
        dist = dist_mod
    return world, rank, local, dist


def max_over_ranks(x: float, dist, device: str = "cuda") -> float:
    """Largest value over all ranks (the slowest replica's step time)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, ms_per_step: float, world: int) -> float:
    """Replicas only: every rank runs the full workload, so the job checks
    world x units per (slowest) step."""
    return units_per_rank * world / (ms_per_step / 1e3)


def _cpu_sample(threads: int, j_first: int, n_extra: int) -> tuple[int, float]:
    """One pass of the CPU sample: the main instance's sets within constraints
    [j_first, 62) at every level |S| <= 6, and the first n_extra extra
    instances to |S| = n under their budget.  Returns (candidates, seconds)."""
    from oracle import oracle as O
    probs, kmax, budget = workload()
    t0 = time.perf_counter()
    n = O.enumerate_tail(probs[0], j_first, k_max=kmax[0], nthreads=threads).n_cand
    for i in range(1, 1 + n_extra):
        n += O.enumerate_sets(probs[i], k_max=kmax[i], budget=budget[i], nthreads=threads, keep_records=False).n_cand
    return n, time.perf_counter() - t0


def cpu_baseline(steps: int = 1, warmup: int = 0, single_core: bool = True) -> dict:
    """The C oracle (restatement of the reference's algorithm) on the host, on
    a bounded sample with the GPU workload's mix: the m = 62 instance at all
    six levels (its active sets within the last 40 constraints, a family
    closed under subsets: every candidate is checked exactly as in the full
    enumeration) plus 3 of the 32 extra instances at their full budget, every
    host thread; beside it one host core on a smaller tail (last 28)."""
    threads = os.cpu_count() or 1
    for _ in range(warmup):
        _cpu_sample(threads, CPU_TAIL_FIRST, CPU_EXTRAS)
    vals, n, secs = [], 0, 0.0
    for _ in range(max(1, steps)):
        n, dt = _cpu_sample(threads, CPU_TAIL_FIRST, CPU_EXTRAS)
        vals.append(n / dt)
        secs = dt
    out = {"value": statistics.median(vals), "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"C oracle: main instance n=12 m=62 p=6, every active set |S|<=6 within constraints "
                     f"{CPU_TAIL_FIRST}..61, plus extra instances 1..{CPU_EXTRAS} of 32 to |S|=n at budget "
                     f"{EXTRA_BUDGET} ({n} candidates per step)",
           "seconds_per_step": secs, "candidates_per_step": n}
    if single_core:
        n1, dt1 = _cpu_sample(1, CPU_TAIL_FIRST_1CORE, 0)
        out["single_core"] = {"value": n1 / dt1, "unit": UNIT, "cores": 1,
                              "sample": f"main instance, every active set |S|<=6 within constraints "
                                        f"{CPU_TAIL_FIRST_1CORE}..61 ({n1} candidates)"}
    return out


def mplp_measure(prec, stream, dev, steps: int = 3) -> dict:
    """The mpLP row (Q = 0): 32 random mpLPs of mixed sizes (``mplp_batch``),
    every instance enumerated to |S| = n, device-resident plan, CUDA events
    around `steps` runs; the plain FP64 path beside it (same regions) and the
    C oracle on the host on the first 8 instances."""
    import torch
    from mpqpcudasolver_gb300 import problems as P
    from mpqpcudasolver_gb300 import solver
    from oracle import oracle as O
    probs = [P.scale_problem(p) for p in P.mplp_batch()]

    def timed(precision):
        plan = solver.Plan(probs, precision=precision, mem_fraction=0.85)
        for _ in range(2):
            plan.run(stream.cuda_stream)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            plan.run(stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        res = plan.results()
        plan.close()
        assert res.status == 0, res.status
        return res, e0.elapsed_time(e1) / steps

    res, ms = timed(prec)
    r64, ms64 = timed(solver.FP64)
    threads = os.cpu_count() or 1
    sample = probs[:8]
    t0 = time.perf_counter()
    n_cpu = sum(O.enumerate_sets(pr, k_max=pr.n, nthreads=threads, keep_records=False).n_cand for pr in sample)
    cpu_s = time.perf_counter() - t0
    return {"workload": "32 random mpLPs (Q = 0; n~U{4..8}, m~U{2n+6..2n+16}, p~U{2..4}, parametric cost), "
                        "all instances to |S| = n",
            "candidates_per_step": res.candidates, "ms_per_step": ms, "value": res.candidates / (ms / 1e3),
            "unit": UNIT, "optimal": res.total("optimal"), "regions": res.total("regions"),
            "fp64_path": {"ms_per_step": ms64, "value": r64.candidates / (ms64 / 1e3),
                          "regions_identical": same_regions(res, r64)},
            "cpu_baseline": {"value": n_cpu / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"C oracle, the first 8 instances to |S| = n ({n_cpu} candidates)"}}


DEFAULT_SETTINGS = dict(tile_w=8, feas_warps=4, feas_chunk=32)
CFG2_BUDGET = 1 << 25      # config 2 (n=10, m=43, p=4) to |S| = 10: the levels that fit this many candidates
CFG5_BUDGET = 1 << 21      # config 5 (64 MPC instances) to |S| = n: per instance


def other_configs(stream, dev) -> dict:
    """The other two GPU configurations of the metric's family, timed in both
    precisions on device-resident plans (CUDA events, one warm and one timed
    run each way), with the regions compared:
    * config 2: the n=10, m=43, p=4 instance, enumerated toward |S| = 10 with
      superset pruning; the levels that fit 2^25 candidates are checked;
    * config 5: 64 condensed MPC instances (seeds 0..63, n=12, m=72, p=4),
      each to |S| = n under a 2^21-candidate budget."""
    import torch
    from mpqpcudasolver_gb300 import problems as P
    from mpqpcudasolver_gb300 import solver
    cases = {"config2_n10_m43_p4": ([P.scale_problem(P.random_n10_m43_p4())], 10, CFG2_BUDGET),
             "config5_mpc64": ([P.scale_problem(p) for p in P.mpc_batch(64)], 12, CFG5_BUDGET)}
    out = {}
    for name, (probs, kmax, bud) in cases.items():
        row = {}
        res = {}
        for prec, tag in ((solver.MIXED, "mixed"), (solver.FP64, "fp64")):
            plan = solver.Plan(probs, precision=prec, k_max=kmax, budget=bud, mem_fraction=0.85)
            plan.run(stream.cuda_stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.run(stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            r = plan.results()
            plan.close()
            ms = e0.elapsed_time(e1)
            res[tag] = r
            row[tag] = {"ms": ms, "value": r.candidates / (ms / 1e3), "unit": UNIT}
        a, b = res["mixed"], res["fp64"]
        row["candidates"] = a.candidates
        row["deepest_level"] = int(a.inst["last_level"].max())
        row["truncated_instances"] = int(a.inst["truncated"].sum())
        row["regions"] = a.total("regions")
        row["regions_identical"] = same_regions(a, b)
        row["speedup_mixed_vs_fp64"] = row["mixed"]["value"] / row["fp64"]["value"]
        out[name] = row
    return out


def settings_compare(stream, dev) -> dict:
    """The autotuner against the fixed default launch settings (8 threads per
    screen LP, 4 LP1 warps per block, 32 candidates per claim) on four batch
    shapes: the bench batch, its main instance alone, 64 MPC instances
    (n=12, m=72, p=4) to |S| <= 4, and 64 small mixed-size problems (n <= 8,
    m <= 30) to |S| = n.  Device time of one full run (graph), the best of
    two, each way."""
    import torch
    from mpqpcudasolver_gb300 import problems as P
    from mpqpcudasolver_gb300 import solver
    probs, kmax, budget = workload()
    mpc = [P.scale_problem(p) for p in P.mpc_batch(64)]
    pop = [P.scale_problem(p) for p in P.pop_like_set(64, seed=0, n_max=8, m_max=30)]
    cases = {"bench_batch": (probs, kmax, budget), "main_instance": (probs[:1], kmax[:1], budget[:1]),
             "mpc64_k4": (mpc, 4, 0), "small64_full_depth": (pop, [p.n for p in pop], 0)}
    out = {}
    for name, (pr, km, bu) in cases.items():
        row = {}
        for how, extra in (("default", DEFAULT_SETTINGS), ("tuned", dict(autotune=1))):
            plan = solver.Plan(pr, precision=solver.MIXED, k_max=km, budget=bu, mem_fraction=0.85, **extra)
            plan.run(stream.cuda_stream)
            best = None
            for _ in range(2):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                plan.run(stream.cuda_stream)
                e1.record(stream)
                torch.cuda.synchronize(dev)
                ms = e0.elapsed_time(e1)
                best = ms if best is None else min(best, ms)
            r = plan.results()
            plan.close()
            row[how] = {"ms": best, "settings": r.settings, "regions": r.total("regions")}
        row["speedup"] = row["default"]["ms"] / row["tuned"]["ms"]
        row["same_regions"] = row["default"]["regions"] == row["tuned"]["regions"]
        out[name] = row
    return out


def basis_sharing_compare(stream, dev) -> dict:
    """LP2 basis sharing (lp2_warm=1: the first-stage dual LP of each set
    starts from its parent's final basis) against the default single-row
    start, on the bench batch: device time of a full run and of the screen's
    first stage (best of two runs each way), first-stage iterations per LP,
    the LPs offered a valid parent basis and those that started from it, and
    the regions compared."""
    import torch
    from mpqpcudasolver_gb300 import solver
    probs, kmax, budget = workload()
    out = {}
    regs = {}
    for how, extra in (("default", {}), ("shared", dict(lp2_warm=1))):
        plan = solver.Plan(probs, precision=solver.MIXED, k_max=kmax, budget=budget, mem_fraction=0.85,
                           **DEFAULT_SETTINGS, **extra)
        plan.run(stream.cuda_stream)
        best, stage0 = None, None
        for _ in range(2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.run(stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            best = e0.elapsed_time(e1) if best is None else min(best, e0.elapsed_time(e1))
            plan.run_timed()
            st = sum(v[0] for kname, v in plan.kernel_times().items()
                     if kname.startswith("k_opt_screen<dual") and kname != "k_opt_screen<dual,rows>")
            stage0 = st if stage0 is None else min(stage0, st)
        r = plan.results()
        plan.close()
        lps = r.total("lp2_first_stage_lps")
        out[how] = {"ms": best, "first_stage_ms": stage0, "first_stage_lps": lps,
                    "iterations_per_lp": r.total("lp2_first_stage_pivots") / max(lps, 1),
                    "offered": r.total("lp2_warm_offered"), "started": r.total("lp2_warm_started")}
        regs[how] = r
    out["regions_identical"] = same_regions(regs["default"], regs["shared"])
    out["speedup"] = out["default"]["ms"] / out["shared"]["ms"]
    return out


def run_reference(args):
    world, rank, local, dist = dist_setup(args.gpus)
    if rank != 0:
        return 0
    # host work: one untimed pass is warm-up enough (no device, no caches to fill)
    cb = cpu_baseline(steps=args.steps, warmup=min(args.warmup, 1))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": cb["seconds_per_step"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_dict("fp64 (CPU)"),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "single_core")},
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    from mpqpcudasolver_gb300 import solver

    world, rank, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    probs, kmax, budget = workload()
    prec = solver.MIXED if args.precision == "mixed" else solver.FP64
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    plan = solver.Plan(probs, precision=prec, k_max=kmax, budget=budget, mem_fraction=0.85, autotune=1)
    for _ in range(args.warmup):
        plan.run(stream.cuda_stream)
    res = plan.results()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for s in range(args.steps):
            if s:
                flush.zero_()
            plan.run_timed(stream.cuda_stream)
        ev1.record(stream)
        torch.cuda.synchronize(dev)
    # kernel times of the last timed step (events on the launching stream)
    kt = plan.kernel_times()
    res = plan.results()
    elapsed = ev0.elapsed_time(ev1)
    ms_step = max_over_ranks(elapsed / args.steps, dist)
    if dist is not None:
        dist.barrier()
    assert res.status == 0, res.status
    cand = res.candidates
    value = whole_job_rate(cand, ms_step, world)
    launches = plan.launches
    settings = res.settings
    plan.close()
    del plan
    torch.cuda.synchronize(dev)

    # plain FP64 path on the same workload: speed-up and identical regions
    fp64 = None
    if prec == solver.MIXED and not args.skip_fp64:
        p64 = solver.Plan(probs, precision=solver.FP64, k_max=kmax, budget=budget, mem_fraction=0.85)
        p64.run(stream.cuda_stream)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        p64.run(stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        r64 = p64.results()
        fp64 = {"ms_per_step": e0.elapsed_time(e1), "candidates": r64.candidates}
        fp64["value"] = r64.candidates / (fp64["ms_per_step"] / 1e3)
        fp64["regions_identical"] = same_regions(res, r64)
        fp64["regions"] = r64.total("regions")
        fp64["optimal"] = r64.total("optimal")
        fp64["feasible_identical"] = r64.total("feasible") == res.total("feasible")
        p64.close()
        del p64

    # end to end through the C ABI: host problem arrays in, host results out
    e2e_vals, h2d, d2h = [], 0, 0
    for _ in range(max(1, args.e2e_steps)):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        r = solver.solve(probs, precision=prec, k_max=kmax, budget=budget, mem_fraction=0.85, autotune=1)
        dt = time.perf_counter() - t0
        e2e_vals.append(r.candidates / dt)
        h2d, d2h = r.h2d_bytes, r.d2h_bytes
    # slowest rank's end-to-end rate, times the replicas
    e2e_val = -max_over_ranks(-statistics.median(e2e_vals), dist) * world

    if rank != 0:
        return 0
    elem = 4 if prec == solver.MIXED else 8
    tname = "float" if prec == solver.MIXED else "double"
    dominant = max(kt.items(), key=lambda kv: kv[1][0])[0] if kt else None
    peaks = measured_peaks()
    peak_src = peaks["source"] + " (MEASURED_PEAKS.json hbm_gbs)"
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    clocks = clk.summary()
    mhz = clocks.get("sm_mhz") or 2070.0

    # LP1, the dominant kernel: HBM roofline on the unique bytes it must move,
    # and the issue roofline beside it (it is issue-bound, not HBM-bound)
    lp1 = f"k_feasibility<{tname}>"
    ms_lp1, nl_lp1 = kt.get(lp1, (0.0, 1))
    nl_lp1 = max(nl_lp1, 1)
    lp1_cand = res.candidates - len(probs)
    ubytes = lp1_unique_bytes(res)
    achieved = ubytes / (ms_lp1 / 1e3) / 1e9 if ms_lp1 > 0 else None
    tr_pc = profile_figure("lp1_traffic.json", "dram_bytes_per_unit")
    ipc = profile_figure("lp1_issue.json", "warp_inst_per_unit")
    issue_ms = ipc * lp1_cand / (sms * 4 * mhz * 1e6) * 1e3 if ipc else None
    roof = {"bound": "hbm", "kernel": lp1, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
            "traffic": tr_pc * lp1_cand / nl_lp1 if tr_pc else None,
            "algorithmic_bytes_per_launch": ubytes / nl_lp1, "units_per_launch": lp1_cand / nl_lp1,
            "avg_launch_ms": ms_lp1 / nl_lp1, "launches_per_step": nl_lp1, "peak_source": peak_src,
            "per_unit": "each distinct parent once (live tableau rows + ids + node), 56 B per candidate, each "
                        "stored child's live rows + ids + 8 B hash slot (device counters of the run)",
            "issue": {"warp_inst_per_candidate": ipc, "ideal_ms_per_step": issue_ms,
                      "frac": (issue_ms / ms_lp1) if (issue_ms and ms_lp1 > 0) else None,
                      "model": "warp instructions per candidate (ncu) x candidates / (SMs x 4 schedulers x "
                               "median SM clock): the time at one instruction per scheduler per cycle"}}
    # the optimality screen (second kernel): time and measured DRAM traffic
    screen = [k for k in kt if k.startswith("k_opt_screen")]
    n_eval = res.total("feasible")
    screen_info = None
    if screen:
        ms_s = sum(kt[k][0] for k in screen)
        sp = profile_figure("opt_traffic.json", "dram_bytes_per_unit")
        si = profile_figure("opt_issue.json", "warp_inst_per_unit")
        s_issue = si * n_eval / (sms * 4 * mhz * 1e6) * 1e3 if si else None
        screen_info = {"kernels": "+".join(screen), "ms_per_step": ms_s, "sets_per_step": n_eval,
                       "dram_gbs": sp * n_eval / (ms_s / 1e3) / 1e9 if sp else None,
                       "issue_frac": (s_issue / ms_s) if s_issue else None}
    cert_ms = kt.get("k_lp1_cert", (0.0, 0))[0]
    opt = res.opt
    errs = opt["err"][np.isfinite(opt["err"])] if len(opt) else np.zeros(0)
    reg = opt[opt["region"] == 1] if len(opt) else opt
    cb = cpu_baseline(steps=1)
    mplp = None if args.skip_mplp else mplp_measure(prec, stream, dev)
    tune_cmp = None if (args.skip_tune_compare or prec != solver.MIXED) else settings_compare(stream, dev)
    others = None if args.skip_configs else other_configs(stream, dev)
    warm_cmp = None if (args.skip_tune_compare or prec != solver.MIXED) else basis_sharing_compare(stream, dev)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64cert" if prec == solver.MIXED else "f64",
        "data": "synthetic (seeded generators)", "config": config_dict(args.precision),
        "candidates_per_step": cand,
        "speedup_vs_fp64": (value / world / fp64["value"]) if fp64 else None,
        "fp64_path": fp64,
        "roofline": roof,
        "lp1_certificate": {"infeasible_certified": res.total("lp1_certified"),
                            "fp64_resolved": res.total("fallback_lp1"),
                            "cert_missed": res.total("lp1_cert_missed"), "ms_per_step": cert_ms},
        "law_error": {"max": float(errs.max()) if errs.size else None,
                      "max_regions": float(np.nanmax(reg["err"])) if len(reg) else None,
                      "results": int(len(opt)),
                      "what": "per optimal set: one FP64 refinement step of its KKT solve, relative to the law"},
        "screen": screen_info,
        "launch_settings": settings,
        "other_configs": {k: {"mixed": v["mixed"]["value"], "fp64": v["fp64"]["value"], "unit": UNIT,
                              "candidates": v["candidates"], "deepest_level": v["deepest_level"],
                              "regions_identical": v["regions_identical"]} for k, v in others.items()}
        if others else None,
        "autotune_vs_default": {k: {"default_ms": v["default"]["ms"], "tuned_ms": v["tuned"]["ms"],
                                    "tuned": v["tuned"]["settings"], "speedup": v["speedup"],
                                    "same_regions": v["same_regions"]} for k, v in tune_cmp.items()}
        if tune_cmp else None,
        "lp2_basis_sharing": {"default_ms": warm_cmp["default"]["ms"], "shared_ms": warm_cmp["shared"]["ms"],
                              "first_stage_ms": [warm_cmp["default"]["first_stage_ms"],
                                                 warm_cmp["shared"]["first_stage_ms"]],
                              "iterations_per_lp": [warm_cmp["default"]["iterations_per_lp"],
                                                    warm_cmp["shared"]["iterations_per_lp"]],
                              "started_share": warm_cmp["shared"]["started"]
                              / max(warm_cmp["shared"]["first_stage_lps"], 1),
                              "regions_identical": warm_cmp["regions_identical"]}
        if warm_cmp else None,
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "single_core")},
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": "mpqp_solve_batch (C ABI): host arrays in, plan + upload + run + download + free"},
        "clocks": clocks,
        "gpu_launches": launches * args.steps,
        "detail": DETAIL_FILE,
    }
    detail = {
        "pivots_per_s": (res.total("lp1_pivots") + res.total("lp2_pivots") + res.total("cheb_pivots"))
        * world / (ms_step / 1e3),
        "regions_per_step": res.total("regions"), "feasible_per_step": res.total("feasible"),
        "fp64_fallbacks": {"lp1": res.total("fallback_lp1"), "lp1_by_vertex_check": res.total("lp1_vertex_checked"),
                           "optimality": res.total("fallback_opt"),
                           "optimality_by_basis_check": res.total("lp2_certified")},
        "kernels_ms_per_step": {k: round(v[0], 3) for k, v in sorted(kt.items(), key=lambda kv: -kv[1][0])},
        "kernel_launches_per_step": {k: v[1] for k, v in kt.items()},
        "dominant_kernel": dominant,
        "screen_model_bytes_per_s": opt_algorithmic_bytes(probs, res, elem) / (ms_step / 1e3),
        "model_bytes_touched_per_s": model_bytes_touched(probs, res, elem) / (ms_step / 1e3),
        "lp1_parents": res.total("lp1_parents"), "lp1_parent_bytes": res.total("lp1_parent_bytes"),
        "lp1_store_bytes": res.total("lp1_store_bytes"),
        "mplp": mplp,
        "other_configs": others,
        "autotune_vs_default": tune_cmp,
        "lp2_basis_sharing": warm_cmp,
    }
    try:
        with open(DETAIL_FILE, "w") as f:
            json.dump(detail, f, indent=1, default=float)
    except OSError:
        pass
    print(json.dumps(line, default=float), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-mplp", action="store_true", help="leave out the mpLP (Q = 0) measurement")
    ap.add_argument("--skip-configs", action="store_true", help="leave out configs 2 and 5")
    ap.add_argument("--skip-tune-compare", action="store_true",
                    help="leave out the autotuned-vs-default launch settings comparison")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
