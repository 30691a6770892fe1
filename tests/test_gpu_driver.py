"""The driver loops (one call per problem, and batched) against the oracle.

A seeded set of problems of mixed sizes stands in for the reference's test
set; every active set up to |S| = n is checked.  The region count of every
problem must equal the oracle's, through the per-problem drop-in ABI
(``mpqp``) and through the batched native interface, with and without the
device row reduction (the oracle then enumerates the problem its own
restatement of the reduction produced).
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import host, problems as P, solver
from oracle import oracle as O
from oracle import preprocess as R

pytestmark = pytest.mark.gpu

SET = P.pop_like_set(16, seed=0)


def _oracle_regions(reduce):
    out = []
    for prob in SET:
        pr = prob
        if reduce:
            pr = solver.apply_row_status(prob, R.reduce_rows(prob))
        pr = P.scale_problem(pr)
        out.append(O.enumerate_sets(pr, k_max=pr.n, nthreads=4).n_region)
    return np.array(out)


@pytest.mark.parametrize("reduce", [False, True])
def test_batched_driver_region_counts(gpu_lib, reduce):
    want = _oracle_regions(reduce)
    for precision in ("mixed", "fp64"):
        res, batches = host.calculate_mpqp_batched(SET, precision=precision, reduce=reduce, max_batch=8)
        print(f"batched {precision} reduce={reduce}: {res[:, 2].sum()*1e3:.1f} ms for {len(SET)} problems "
              f"in {len(batches)} batches")
        assert sum(batches) == len(SET)
        assert np.array_equal(res[:, 1].astype(int), want), (precision, res[:, 1], want)


def test_per_problem_driver_region_counts(gpu_lib):
    want = _oracle_regions(True)
    res, raw = host.calculate_mpqp_with_CUDA(SET, precision="fp64", reduce=True, reserved_memory=512)
    print(f"per-problem fp64: {res[:, 2].sum()*1e3:.1f} ms for {len(SET)} problems")
    assert np.array_equal(res[:, 1].astype(int), want)
