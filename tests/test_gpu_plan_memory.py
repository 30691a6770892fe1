"""Plans on pooled device memory: no hash clearing between plans.

A plan takes its buffers from a per-device pool that keeps freed memory, and
its subset-test hash is never cleared: each slot's tag comes from the run's
epoch (one counter per device, so no two runs of any plans share one) and
the level, so another plan's entries (or any other leftover bytes) read as
empty slots.  Here plans of different problems run
back to back on the same pooled memory, and a repeated problem must give the
same candidates, pruned and feasible counts and the same feasible, optimal and
region sets as its first run; after the pool is released the same holds.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver

pytestmark = pytest.mark.gpu

FIELDS = ("candidates", "pruned", "feasible", "optimal", "regions", "feasible_digest", "optimal_digest",
          "region_digest")


def _same(a, b):
    for f in FIELDS:
        assert np.array_equal(a.inst[f], b.inst[f]), f


@pytest.mark.parametrize("precision", [solver.MIXED, solver.FP64])
def test_plans_back_to_back_on_pooled_memory(gpu_lib, precision):
    a = [P.scale_problem(P.random_n12_m62_p6())]
    b = [P.scale_problem(P.batch_member(s)) for s in (4, 9, 13)]
    c = [P.scale_problem(P.mpc_mpqp(s)) for s in range(6)]
    kw = dict(precision=precision, cand_cap=1 << 23, arena_bytes=1 << 30)
    ra = solver.solve(a, k_max=4, **kw)
    rb = solver.solve(b, k_max=4, **kw)
    rc = solver.solve(c, k_max=4, **kw)
    # the same problems again, in another order, on the memory the others left
    rc2 = solver.solve(c, k_max=4, **kw)
    ra2 = solver.solve(a, k_max=4, **kw)
    rb2 = solver.solve(b, k_max=4, **kw)
    for r in (ra, rb, rc, ra2, rb2, rc2):
        assert r.status == 0 and r.overflow == 0
    _same(ra, ra2)
    _same(rb, rb2)
    _same(rc, rc2)
    # a plan run several times reuses its own hash across epochs
    plan = solver.Plan(b, precision=precision, k_max=4, cand_cap=1 << 23, arena_bytes=1 << 30)
    for _ in range(3):
        plan.run()
        _same(rb, plan.results())
    plan.close()
    # and after the pool gave its memory back
    gpu_lib.mpqp_release_cached_memory()
    _same(ra, solver.solve(a, k_max=4, **kw))
    print("back-to-back plans: candidates", ra.candidates, rb.candidates, rc.candidates)
