"""CPU restatement of the constraint reduction (test infrastructure only).

The reference's ``MPQPProb.process_constraints`` (``utils.py:163-190``) calls
three functions of ppopt 1.5.1 (a dependency that is not in the reference
tree and not installed here): ``process_program_constraints`` (zero and
duplicate rows), ``find_implicit_equalities`` (a row of [A -F | b] that is the
negation of another makes the pair an equality; one row is kept) and
``find_redundant_constraints`` on ``[A -F; 0 At] u <= [b; bt]`` (an LP per row:
the row is redundant when the other rows already imply it).  This module
restates those steps with numpy and scipy's HiGHS, with the same thresholds
as ``mpqp_reduce_constraints``:

* rows are divided by the 2-norm of their ``[A -F]`` (or ``At``) part; a part
  of norm <= 1e-12 is a zero row;
* two rows (b included) of the same block within a squared distance of 1e-16
  are duplicates, the earlier one is kept;
* a row of A within 1e-16 of the negation of an earlier kept row is dropped and
  the earlier row becomes an equality;
* every other row i is redundant when ``max a_i u`` over all rows that are
  neither zero nor duplicates, with row i relaxed by 1, is at most
  ``d_i + 1e-9``.

Parity with ppopt itself is unpinned (ppopt cannot run here); the tests pin
this restatement on problems with planted zero, duplicate, equality and
redundant rows, whose statuses are known by construction.
"""
from __future__ import annotations

import numpy as np
from scipy.optimize import linprog

ROW_KEPT, ROW_ZERO, ROW_DUPLICATE, ROW_EQUALITY_PAIR, ROW_REDUNDANT, ROW_EQUALITY = range(6)
ZERO_NORM = 1e-12
SAME_ROW = 1e-16
REDUNDANT_TOL = 1e-9


def reduce_rows(prob) -> np.ndarray:
    """Status code per row of A, then per row of CRA (same codes as the C API)."""
    A, b, F = prob.A, np.asarray(prob.b).ravel(), prob.F
    At, bt = prob.CRA, np.asarray(prob.CRb).ravel()
    m, n = A.shape
    p = F.shape[1]
    R = m + At.shape[0]
    a = np.zeros((R, n + p))
    a[:m, :n] = A
    a[:m, n:] = -F
    a[m:, n:] = At
    d = np.concatenate([b, bt]).astype(np.float64)
    status = np.full(R, ROW_KEPT, dtype=np.int64)
    norms = np.sqrt(np.sum(a * a, axis=1))
    for r in range(R):
        if not norms[r] > ZERO_NORM:
            status[r] = ROW_ZERO
        else:
            a[r] /= norms[r]
            d[r] /= norms[r]

    def dist2(r, s, sign):
        return float(np.sum((a[r] - sign * a[s]) ** 2) + (d[r] - sign * d[s]) ** 2)

    for r in range(R):
        if status[r] != ROW_KEPT:
            continue
        for s in range(0 if r < m else m, r):
            if status[s] not in (ROW_ZERO, ROW_DUPLICATE) and dist2(r, s, 1.0) < SAME_ROW:
                status[r] = ROW_DUPLICATE
                break
    for r in range(m):
        if status[r] != ROW_KEPT:
            continue
        for s in range(r):
            if status[s] in (ROW_KEPT, ROW_EQUALITY) and dist2(r, s, -1.0) < SAME_ROW:
                status[r] = ROW_EQUALITY_PAIR
                status[s] = ROW_EQUALITY
                break
    lp = [r for r in range(R) if status[r] not in (ROW_ZERO, ROW_DUPLICATE)]
    M, dd = a[lp], d[lp]
    for idx, r in enumerate(lp):
        if status[r] != ROW_KEPT:
            continue
        rhs = dd.copy()
        rhs[idx] += 1.0
        res = linprog(-M[idx], A_ub=M, b_ub=rhs, bounds=[(None, None)] * M.shape[1], method="highs")
        if res.status == 0 and -res.fun <= dd[idx] + REDUNDANT_TOL:
            status[r] = ROW_REDUNDANT
    return status


def planted_problem(seed: int = 0):
    """A random mpQP with rows whose reduction status is known by construction.

    Base: ``random_mpqp(n=4, m=10, p=2)``.  Appended rows of A (in this order):
    a zero row (b = 1), a copy of row 2 scaled by 2.5 (duplicate), a row equal
    to 0.5 (row 0 + row 1) with b raised by 0.3 (strictly redundant: implied by
    rows 0 and 1), an implicit-equality pair through the origin (a, b = 0 and
    its negation), and a copy of row 5 scaled by 0.25 with b raised by 2
    (parallel and looser: redundant).  CRA gets a duplicate of its first row
    and a looser copy of its second (redundant).  Returns (prob, expected)
    where ``expected`` maps row index -> status for the planted rows.
    """
    from mpqpcudasolver_gb300 import problems as P
    base = P.random_mpqp(4, 10, 2, seed=seed)
    rng = np.random.default_rng(1000 + seed)
    A, b, F = base.A, base.b, base.F
    m = A.shape[0]
    rows_A, rows_b, rows_F = [], [], []
    rows_A.append(np.zeros(4)); rows_b.append(1.0); rows_F.append(np.zeros(2))              # m: zero
    rows_A.append(2.5 * A[2]); rows_b.append(2.5 * b[2]); rows_F.append(2.5 * F[2])       # m+1: duplicate
    rows_A.append(0.5 * (A[0] + A[1])); rows_b.append(0.5 * (b[0] + b[1]) + 0.3)          # m+2: redundant
    rows_F.append(0.5 * (F[0] + F[1]))
    e = rng.standard_normal(4); e /= np.linalg.norm(e); g = rng.normal(0.0, 0.5, 2)
    rows_A.append(e); rows_b.append(0.0); rows_F.append(g)                                 # m+3: equality
    rows_A.append(-e); rows_b.append(0.0); rows_F.append(-g)                               # m+4: its pair
    rows_A.append(0.25 * A[5]); rows_b.append(0.25 * b[5] + 2.0); rows_F.append(0.25 * F[5])  # m+5: redundant
    prob = base.copy()
    prob.A = np.vstack([A, np.array(rows_A)])
    prob.b = np.concatenate([b, np.array(rows_b)])
    prob.F = np.vstack([F, np.array(rows_F)])
    prob.CRA = np.vstack([base.CRA, 3.0 * base.CRA[0], base.CRA[1]])
    prob.CRb = np.concatenate([base.CRb, [3.0 * base.CRb[0], base.CRb[1] + 0.5]])
    prob.name = f"planted(seed={seed})"
    mt = prob.A.shape[0]
    expected = {m: ROW_ZERO, m + 1: ROW_DUPLICATE, m + 2: ROW_REDUNDANT, m + 3: ROW_EQUALITY,
                m + 4: ROW_EQUALITY_PAIR, m + 5: ROW_REDUNDANT,
                mt + base.CRA.shape[0]: ROW_DUPLICATE, mt + base.CRA.shape[0] + 1: ROW_REDUNDANT}
    for name in ("A", "b", "F", "CRA", "CRb"):
        setattr(prob, name, np.ascontiguousarray(getattr(prob, name), dtype=np.float64))
    return prob, expected
