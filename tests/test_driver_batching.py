"""Host logic of the batched driver: memory-bounded batches that split on overflow.

The device is replaced by a fake ``solver.solve`` that fails with
MPQP_ECAPACITY whenever a batch holds more than three problems, and reports
one region per variable otherwise; the driver must split down to batches of
at most three, keep every problem's result in its own row, and re-raise when
a single problem does not fit.
"""
import numpy as np
import pytest

from mpqpcudasolver_gb300 import host, problems as P, solver


class _Res:
    def __init__(self, probs):
        self.inst = np.array([(pr.n, 10 * pr.m) for pr in probs], dtype=[("regions", "i8"), ("candidates", "i8")])


def _fake(limit):
    calls = []

    def solve(probs, precision=None, k_max=None, mem_fraction=None, **kw):
        calls.append(len(probs))
        if len(probs) > limit:
            raise solver.MpqpError(solver.ECAPACITY, "fake overflow")
        return _Res(probs)
    return solve, calls


def test_batches_split_until_they_fit(monkeypatch):
    import torch
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda: (8 << 30, 16 << 30))
    fake, calls = _fake(3)
    monkeypatch.setattr(solver, "solve", fake)
    probs = P.pop_like_set(11, seed=3)
    res, batches = host.calculate_mpqp_batched(probs, max_batch=8, reserved_memory=1024)
    assert max(batches) <= 3 and sum(batches) == len(probs)
    assert [int(r[0]) for r in res] == list(range(len(probs)))
    assert [int(r[1]) for r in res] == [pr.n for pr in probs]
    assert [int(r[3]) for r in res] == [10 * pr.m for pr in probs]


def test_single_problem_that_does_not_fit_raises(monkeypatch):
    import torch
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda: (8 << 30, 16 << 30))
    fake, _ = _fake(0)
    monkeypatch.setattr(solver, "solve", fake)
    with pytest.raises(solver.MpqpError):
        host.calculate_mpqp_batched(P.pop_like_set(2, seed=1), max_batch=2)
