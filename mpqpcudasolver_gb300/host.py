"""Python host side, mirroring the reference's driver interface for this path.

The reference's driver (``main.py``) preprocesses each problem with
``MPQPProb`` (``utils.py:147-229``), builds two standard-form LPs
(``main.py:87-137``), calls ``mpqp_cuda.so:mpqp`` through ctypes
(``main.py:144``) and turns the returned active sets into critical regions
(``utils.py:23-144``).  This module keeps those names, argument meanings and
error behaviour, with libmpqp_gb300.so behind the ctypes boundary:

* ``MPQPProb``               -- ``utils.py:147-229`` without the ppopt steps
* ``build_lp_data``          -- ``main.py:87-137`` (same matrices, same layout)
* ``load_mpqp_cuda``         -- ``main.py:12-50`` (same argtypes / restype)
* ``calculate_mpqp_with_CUDA`` -- ``main.py:11-173`` for a list of problems
* ``active_sets_to_regions`` -- ``utils.py:128-144``; the laws and region rows
  are computed on the device (FP64) instead of with numpy + Gurobi.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import solver
from .problems import MPQP, scale_problem


class MPQPProb:
    """Problem holder of ``utils.py:147-161``.

    ``process_constraints`` applies the reference's numerical scaling
    (``utils.py:192-229``).  With ``reduce=True`` it first runs the row
    reduction that the reference takes from ppopt (zero and duplicate rows,
    implicit equalities, redundant rows; ``utils.py:165-190``) on the device
    (``mpqp_reduce_constraints``); the default keeps every row, as the golden
    fixtures of the reference's own driver were made without ppopt.
    """

    def __init__(self, A, b, c, H, Q, CRa, CRb, F):
        self.A = np.asarray(A, dtype=np.float64)
        self.b = np.asarray(b, dtype=np.float64).reshape(-1, 1)
        self.c = np.asarray(c, dtype=np.float64).reshape(-1, 1)
        self.H = np.asarray(H, dtype=np.float64)
        self.Q = np.asarray(Q, dtype=np.float64)
        self.inv_Q = np.linalg.pinv(self.Q)
        self.A_t = np.asarray(CRa, dtype=np.float64)
        self.b_t = np.asarray(CRb, dtype=np.float64).reshape(-1, 1)
        self.F = np.asarray(F, dtype=np.float64)
        self.equality_indices = []
        self.num_x = self.A.shape[1]
        self.n_active_sets = 0

    @classmethod
    def from_mpqp(cls, prob: MPQP) -> "MPQPProb":
        return cls(prob.A, prob.b, prob.c, prob.H, prob.Q, prob.CRA, prob.CRb, prob.F)

    def to_mpqp(self) -> MPQP:
        return MPQP(self.Q.copy(), self.c.ravel().copy(), self.H.copy(), self.A.copy(), self.b.ravel().copy(),
                    self.F.copy(), self.A_t.copy(), self.b_t.ravel().copy())

    def process_constraints(self, scale_method: int = 1, reduce: bool = False):
        if reduce:
            from .solver import reduce_constraints
            _, red = reduce_constraints(self.to_mpqp())
            self.A, self.F, self.b = red.A, red.F, red.b.reshape(-1, 1)
            self.A_t, self.b_t = red.CRA, red.CRb.reshape(-1, 1)
            self.equality_indices = list(red.meta["equality_rows"])
        if scale_method == 2:
            H = np.block([self.A, -self.F])
            norm = np.linalg.norm(H, axis=1, keepdims=True)
            self.A, self.b, self.F = self.A / norm, self.b / norm, self.F / norm
        if scale_method == 1:
            s = scale_problem(self.to_mpqp())
            self.A, self.F, self.b = s.A, s.F, s.b.reshape(-1, 1)
            self.A_t, self.b_t = s.CRA, s.CRb.reshape(-1, 1)
            self.Q, self.H, self.c = s.Q, s.H, s.c.reshape(-1, 1)
        self.inv_Q = np.linalg.pinv(self.Q)


def build_lp_data(prog: MPQPProb) -> dict:
    """The LP1 / LP2 matrices of ``main.py:87-128`` (same shapes, signs, bases)."""
    num_c, num_x = prog.A.shape
    n_eqs = num_c + num_x
    num_cp, num_t = prog.A_t.shape
    A1 = np.vstack((np.hstack((prog.A, -prog.F)), np.hstack((np.zeros((num_cp, num_x)), prog.A_t))))
    M1 = A1.shape[0]
    A1 = np.hstack((A1, -A1.sum(axis=1, keepdims=True), np.eye(M1)))
    N1 = A1.shape[1]
    xb1 = np.vstack((prog.b, prog.b_t))
    A0 = A1[:num_c, :num_x].T
    A2 = np.vstack((
        np.hstack((np.zeros((num_c, num_x + num_t)), -np.eye(num_c), np.ones((num_c, 1)))),
        np.hstack((np.zeros(num_x + num_t + num_c), -1)),
        np.hstack((np.zeros((num_cp, num_x)), prog.A_t, np.zeros((num_cp, num_c + 1)))),
        np.hstack((prog.Q, prog.H, prog.A.T, np.zeros((num_x, 1)))),
        np.hstack((prog.A, -prog.F, np.eye(num_c), np.zeros((num_c, 1))))))
    xb2 = np.vstack((np.zeros((num_c + 1, 1)), prog.b_t, -prog.c, prog.b))
    neg = xb2[:, 0] < 0
    xb2[neg] = -xb2[neg]
    A2[neg, :] = -A2[neg, :]
    M2 = A2.shape[0]
    A2 = np.hstack((A2, -A2[:, :num_x + num_t].sum(axis=1, keepdims=True), np.eye(M2)))
    N2 = A2.shape[1]
    b1 = np.arange(N1 - M1, N1, dtype=np.intc)
    b2 = np.hstack((np.arange(num_x), np.arange(num_x + num_t, num_x + num_t + num_c),
                    np.arange(N2 - M2, N2 - n_eqs))).astype(np.intc)
    non_b2 = np.setdiff1d(np.arange(0, N2, dtype=np.intc), b2)
    return dict(A0=np.asfortranarray(A0), A1=np.asfortranarray(A1), xb1=np.ascontiguousarray(xb1),
                b1=b1, M1=M1, N1=N1, A2=np.asfortranarray(A2), xb2=np.ascontiguousarray(xb2), b2=b2,
                non_b2=non_b2.astype(np.intc), M2=M2, N2=N2, n_eqs=n_eqs, num_c=num_c, num_x=num_x,
                num_t=num_t)


def load_mpqp_cuda():
    """``ctypes`` binding exactly as ``main.py:25-50`` declares it."""
    lib = ctypes.cdll.LoadLibrary(solver.library_path())
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    lib.mpqp.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                         dp, dp, ip, ctypes.c_int, ctypes.c_int, dp, dp, ip, ip, ctypes.c_int, ctypes.c_int,
                         ctypes.c_int, ctypes.c_int]
    lib.mpqp.restype = ctypes.POINTER(solver.GPUResults)
    lib.mpqp_free.argtypes = [ctypes.POINTER(solver.GPUResults)]
    return lib


def call_mpqp(lib, d: dict, k_min: int = 0, k_max: int | None = None, extra_batches: int = 0,
              reserved_memory: int = 0):
    """The call of ``main.py:130-144`` on the matrices of ``build_lp_data``."""
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    k_max = d["num_x"] if k_max is None else k_max
    return lib.mpqp(d["A0"].ctypes.data_as(dp), d["num_c"], d["num_x"], d["num_t"], k_min, k_max, extra_batches,
                    d["A1"].ctypes.data_as(dp), d["xb1"].ctypes.data_as(dp), d["b1"].ctypes.data_as(ip),
                    d["M1"], d["N1"], d["A2"].ctypes.data_as(dp), d["xb2"].ctypes.data_as(dp),
                    d["b2"].ctypes.data_as(ip), d["non_b2"].ctypes.data_as(ip), d["M2"], d["N2"], d["n_eqs"],
                    reserved_memory)


def decode_active_sets(all_active_sets, n_sets: int, num_x: int) -> list[list[int]]:
    """-1 padded rows -> lists (``utils.py:108-116``)."""
    out = []
    for i in range(n_sets):
        s = []
        for e in range(num_x):
            v = all_active_sets[i * num_x + e]
            if v == -1:
                break
            s.append(int(v))
        out.append(s)
    return out


def active_sets_to_regions(prog: MPQPProb, all_active_sets, is_region=None) -> list[dict]:
    """``utils.py:128-144``: one region dict per active set whose Chebyshev
    radius is at least 1e-8.  Laws and normalised region rows come from the
    device in FP64.  ``is_region`` (optional, e.g. ``GPUResults.is_region``):
    the radius test ``mpqp()`` already ran for these sets; without it the
    device computes each set's radius with its laws (``mpqp_critical_regions``).
    Neither way enumerates any set."""
    sets = decode_active_sets(all_active_sets, prog.n_active_sets, prog.num_x)
    if not sets:
        return []
    prob = prog.to_mpqp()
    if is_region is not None:
        laws = solver.region_laws(prob, sets)
        keep = [bool(is_region[i]) for i in range(len(sets))]
    else:
        laws = solver.region_laws(prob, sets, with_radius=True)
        keep = [law is not None and law["r"] >= 1e-8 for law in laws]
    return [law for law, k in zip(laws, keep) if law is not None and k]


def calculate_mpqp_with_CUDA(problems, precision: str = "mixed", reduce: bool = False, reserved_memory: int = 0):
    """``main.py:11-173`` over a list of ``MPQP`` problems, one call each.

    Returns rows (index, n_regions, total_time, time_GPU) like the reference,
    plus the raw results.  ``precision`` selects the FP32 kernels with FP64
    certificates ("mixed", the default of ``mpqp()``) or the plain FP64
    kernels ("fp64"; environment variable MPQP_PRECISION);
    ``reduce`` runs the device row reduction first (the ppopt steps of
    ``utils.py:165-190``); ``reserved_memory`` (MiB) is the argument of
    ``main.py:144``: device memory left free when the call sizes its buffers.
    """
    import os
    os.environ["MPQP_PRECISION"] = "mixed" if precision == "mixed" else "fp64"
    lib = load_mpqp_cuda()
    lib.warm_up()
    results = np.zeros((len(problems), 4))
    raw = []
    for idx, prob in enumerate(problems):
        prog = MPQPProb.from_mpqp(prob)
        prog.process_constraints(scale_method=1, reduce=reduce)
        d = build_lp_data(prog)
        t0 = time.time()
        r = call_mpqp(lib, d, reserved_memory=reserved_memory)
        g = r.contents
        if g.status != 0:
            raise solver.MpqpError(g.status, solver.last_error())
        total = time.time() - t0
        n_final = g.n_final_lps
        sets = decode_active_sets(g.active_sets, n_final, d["num_x"])
        n_regions = int(sum(g.is_region[i] for i in range(n_final)))
        raw.append(dict(sets=sets, n_feasible=g.n_feasible_lps, n_final=n_final, n_regions=n_regions,
                        radius=[g.radius[i] for i in range(n_final)], n_candidates=g.n_candidates))
        results[idx] = (idx, n_regions, total, g.time_GPU)
    return results, raw


def calculate_mpqp_batched(problems, precision: str = "mixed", reduce: bool = False, reserved_memory: int = 0,
                           max_batch: int = 64):
    """The driver loop of ``main.py:52-173`` for many problems at once.

    Each problem is reduced (``reduce``) and scaled as in
    ``MPQPProb.process_constraints``; then up to ``max_batch`` problems share one
    launch sequence (``mpqp_solve_batch``), every active set up to |S| = n.  A
    batch may use the free device memory minus ``reserved_memory`` MiB; a batch
    whose buffers overflow (MPQP_ECAPACITY) is split in half and run again, down
    to single problems (which then raise).

    Returns rows (index, n_regions, time, n_candidates): the time of a batch is
    shared among its problems in proportion to their candidates.
    """
    import torch
    prec = solver.MIXED if precision == "mixed" else solver.FP64
    progs = []
    for prob in problems:
        prog = MPQPProb.from_mpqp(prob)
        prog.process_constraints(scale_method=1, reduce=reduce)
        progs.append(prog.to_mpqp())
    free = torch.cuda.mem_get_info()[0]
    frac = max(0.02, min(0.9, (free - reserved_memory * (1 << 20)) / free))
    results = np.zeros((len(problems), 4))
    batches = []

    def run(idx):
        t0 = time.time()
        try:
            r = solver.solve([progs[i] for i in idx], precision=prec, k_max=[progs[i].n for i in idx],
                             mem_fraction=frac)
        except solver.MpqpError as e:
            if e.code == solver.ECAPACITY and len(idx) > 1:
                half = len(idx) // 2
                run(idx[:half])
                run(idx[half:])
                return
            raise
        dt = time.time() - t0
        cand = np.array([r.inst[j]["candidates"] for j in range(len(idx))], dtype=np.float64)
        share = cand / max(cand.sum(), 1.0)
        for j, i in enumerate(idx):
            results[i] = (i, r.inst[j]["regions"], dt * share[j], cand[j])
        batches.append(len(idx))

    for b0 in range(0, len(problems), max_batch):
        run(list(range(b0, min(b0 + max_batch, len(problems)))))
    return results, batches
