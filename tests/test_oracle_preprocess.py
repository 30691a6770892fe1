"""The CPU restatement of the row reduction, pinned on planted rows.

ppopt (whose steps ``utils.py:165-190`` calls) cannot run here, so the
restatement is pinned by construction: each planted row -- a zero row, a
scaled copy, a convex combination with a raised right-hand side, an
implicit-equality pair through the origin, a looser parallel copy, and the
same kinds in CRA -- must get the status it was built to have.
"""
import numpy as np
import pytest

from oracle import preprocess as R


@pytest.mark.parametrize("seed", range(4))
def test_planted_rows_get_their_status(seed):
    prob, expected = R.planted_problem(seed)
    status = R.reduce_rows(prob)
    assert len(status) == prob.A.shape[0] + prob.CRA.shape[0]
    for row, want in expected.items():
        assert status[row] == want, (row, status[row], want)


def test_generic_random_problem_keeps_every_row():
    from mpqpcudasolver_gb300 import problems as P
    status = R.reduce_rows(P.random_n10_m43_p4())
    assert np.all(status == R.ROW_KEPT)
