"""Verdicts from the reference's own LP formulations, solved with HiGHS.

Test infrastructure only.  This module restates, matrix for matrix, what the
reference builds and solves for one candidate active set S, with
``scipy.optimize.linprog(method="highs")`` standing in for the batched GPU
simplex (whose source exists) and for Gurobi (used for the Chebyshev LP):

* LP1 (feasibility): the standard-form matrix of ``main.py:91-98`` with the
  slack basis of ``main.py:121``, cost 1 on the slack columns of the active
  constraints (``batched_simplex.cu:26-36``); verdict z* <= tol
  (``batched_simplex.cu:308-314`` uses |z| <= 1e-12).
* LP2 (optimality): the matrix of ``main.py:102-118`` (including the row sign
  flips of ``main.py:112-114`` and the shift column of ``main.py:117``),
  specialised to S as ``initialise_A_kernel_1`` does
  (``batched_simplex.cu:635-650``); the last n_c + n_x rows are equalities
  (their slack columns are the artificials of phase 1,
  ``batched_simplex.cu:690-700``); phase 2 minimises -t
  (``batched_simplex.cu:243-254``) over the non-artificial columns.
* Region: ``compute_critical_region`` (``utils.py:23-97``) line by line, with
  HiGHS solving the Chebyshev LP of ``utils.py:62-81``.

It is independent of the C oracle (different formulation, different LP
solver) and is used to check that the C oracle decides the same verdicts.
"""
from __future__ import annotations

import numpy as np
from scipy.optimize import linprog


def build_lp_matrices(prob):
    """LP1/LP2 exactly as ``main.py:87-128`` builds them (column-major not needed here)."""
    A, b, F, Q, H, c = prob.A, prob.b.reshape(-1, 1), prob.F, prob.Q, prob.H, prob.c.reshape(-1, 1)
    A_t, b_t = prob.CRA, prob.CRb.reshape(-1, 1)
    num_c, num_x = A.shape
    n_eqs = num_c + num_x
    num_cp, num_t = A_t.shape
    A1_1 = np.hstack((A, -F))
    A1_2 = np.hstack((np.zeros((num_cp, num_x)), A_t))
    A1 = np.vstack((A1_1, A1_2))
    M1 = A1.shape[0]
    A1 = np.hstack((A1, -A1.sum(axis=1, keepdims=True), np.eye(M1)))
    N1 = A1.shape[1]
    xb1 = np.vstack((b, b_t))
    A0 = A1[:num_c, :num_x].T
    A2_1 = np.hstack((np.zeros((num_c, num_x + num_t)), -np.eye(num_c), np.ones((num_c, 1))))
    A2_2 = np.hstack((np.zeros(num_x + num_t + num_c), -1))
    A2_3 = np.hstack((np.zeros((num_cp, num_x)), A_t, np.zeros((num_cp, num_c + 1))))
    A2_4 = np.hstack((Q, H, A.T, np.zeros((num_x, 1))))
    A2_5 = np.hstack((A, -F, np.eye(num_c), np.zeros((num_c, 1))))
    A2 = np.vstack((A2_1, A2_2, A2_3, A2_4, A2_5))
    xb2 = np.vstack((np.zeros((num_c + 1, 1)), b_t, -c, b))
    neg_idx = xb2[:, 0] < 0
    xb2[neg_idx] = -xb2[neg_idx]
    A2[neg_idx, :] = -A2[neg_idx, :]
    M2 = A2.shape[0]
    A2 = np.hstack((A2, -A2[:, :num_x + num_t].sum(axis=1, keepdims=True), np.eye(M2)))
    N2 = A2.shape[1]
    b1 = np.arange(N1 - M1, N1, dtype=np.intc)
    b2_1 = np.arange(num_x)
    b2_2 = np.arange(num_x + num_t, num_x + num_t + num_c)
    b2_3 = np.arange(N2 - M2, N2 - n_eqs)
    b2 = np.hstack((b2_1, b2_2, b2_3)).astype(np.intc)
    non_b2 = np.setdiff1d(np.arange(0, N2, dtype=np.intc), b2)
    return dict(A0=A0, A1=A1, xb1=xb1, b1=b1, M1=M1, N1=N1, A2=A2, xb2=xb2, b2=b2, non_b2=non_b2,
                M2=M2, N2=N2, n_eqs=n_eqs, n_c=num_c, n_x=num_x, n_t=num_t, n_cp=num_cp)


def lp1_value(mats, S):
    """min sum_{i in S} w_i over the LP1 standard form; returns z* (or nan)."""
    A1, xb1, M1, N1 = mats["A1"], mats["xb1"][:, 0], mats["M1"], mats["N1"]
    K = N1 - M1
    cost = np.zeros(N1)
    for i in S:
        cost[K + i] = 1.0
    res = linprog(cost, A_eq=A1, b_eq=xb1, bounds=(0, None), method="highs")
    return res.fun if res.status == 0 else np.nan


def lp2_value(mats, S):
    """max t over the specialised LP2; returns t* (-inf when infeasible)."""
    A2 = mats["A2"].copy()
    n_c, n_x, n_t, M2, N2, n_eqs = (mats[k] for k in ("n_c", "n_x", "n_t", "M2", "N2", "n_eqs"))
    Sset = set(int(s) for s in S)
    for j in range(n_c):
        col = n_x + n_t + j
        if j in Sset:
            A2[M2 - n_c + j, col] = 0.0
        else:
            A2[M2 - n_c - n_x:M2 - n_c, col] = 0.0
    N_ = N2 - n_eqs
    cost = np.zeros(N_)
    cost[N2 - M2 - 2] = -1.0
    res = linprog(cost, A_eq=A2[:, :N_], b_eq=mats["xb2"][:, 0], bounds=(0, None), method="highs")
    if res.status == 2:
        return -np.inf
    if res.status == 3:
        return np.inf
    return -res.fun if res.status == 0 else np.nan


def scale_constraint(A, b):
    norm_val = 1.0 / np.linalg.norm(A, axis=1, keepdims=True)
    return [A * norm_val, b * norm_val]


def compute_critical_region(A, b, c, H, inv_Q, F, CRA, CRb, active_set, zero_tol=None):
    """``utils.py:23-97`` with HiGHS in place of Gurobi; also returns r*.

    zero_tol=None keeps the reference's exact zero-row test; a number uses the
    relative test max|row| <= zero_tol * max(1, |rhs|) instead."""
    num_t = CRA.shape[1]
    active_set = list(active_set)
    aux = A[active_set] @ inv_Q
    auxinv = np.linalg.pinv(aux @ A[active_set].T)
    inactive = [i for i in range(A.shape[0]) if i not in active_set]
    lagrange_A = -auxinv @ (aux @ H + F[active_set])
    lagrange_b = -auxinv @ (b[active_set] + aux @ c)
    aux = inv_Q @ A[active_set].T
    parameter_A = -aux @ lagrange_A - inv_Q @ H
    parameter_b = -aux @ lagrange_b - inv_Q @ c
    lambda_A, lambda_b = -lagrange_A[0:], lagrange_b[0:]
    inactive_A = A[inactive] @ parameter_A - F[inactive]
    inactive_b = b[inactive] - A[inactive] @ parameter_b
    if zero_tol is None:
        lamba_nonzeros = [i for i, t in enumerate(lambda_A) if np.nonzero(t)[0].shape[0] > 0]
        ineq_nonzeros = [i for i, t in enumerate(inactive_A) if np.nonzero(t)[0].shape[0] > 0]
    else:
        lamba_nonzeros = [i for i, t in enumerate(lambda_A)
                          if np.max(np.abs(t)) > zero_tol * max(1.0, abs(float(np.ravel(lambda_b[i])[0])))]
        ineq_nonzeros = [i for i, t in enumerate(inactive_A)
                         if np.max(np.abs(t)) > zero_tol * max(1.0, abs(float(np.ravel(inactive_b[i])[0])))]
    CR_A = np.vstack((lambda_A[lamba_nonzeros], inactive_A[ineq_nonzeros], CRA))
    CR_b = np.vstack((lambda_b[lamba_nonzeros], inactive_b[ineq_nonzeros], CRb))
    CR_As, CR_bs = scale_constraint(CR_A, CR_b)
    const_norm = np.linalg.norm(CR_As, axis=1, keepdims=True)[:, :1]
    CR_cs = np.zeros((num_t + 1, 1))
    CR_cs[num_t][0] = -1
    A_ball = np.block([[CR_As, const_norm], [CR_cs.T]])
    b_ball = np.concatenate((CR_bs, np.zeros((1, 1))))
    cost = np.zeros(num_t + 1)
    cost[-1] = -1.0
    res = linprog(cost, A_ub=A_ball, b_ub=b_ball.flatten(), bounds=(None, None), method="highs")
    r = res.x[-1] if res.status == 0 else np.nan
    region = None
    if res.status == 0 and not r < 1e-8:
        region = dict(parameter_A=parameter_A, parameter_b=parameter_b, lagrange_A=lagrange_A,
                      lagrange_b=lagrange_b, CR_As=CR_As, CR_bs=CR_bs, active_set=active_set)
    return region, r


def region_for(prob, S, zero_tol=None):
    """Region of S on an MPQP problem (b, c, CRb as column vectors, utils.py:128-144)."""
    inv_Q = np.linalg.pinv(prob.Q)
    return compute_critical_region(prob.A, prob.b.reshape(-1, 1), prob.c.reshape(-1, 1), prob.H,
                                   inv_Q, prob.F, prob.CRA, prob.CRb.reshape(-1, 1), list(S), zero_tol=zero_tol)
