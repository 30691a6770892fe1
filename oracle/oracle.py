"""ctypes front end of the C oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, as the checker.  The product library never
imports it.  ``build()`` compiles ``mpqp_oracle.c`` in place with
``-ffp-contract=off`` so every multiply-add is the explicit ``fma`` the source
spells out (the FP64 device kernels follow the same order).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mpqp_oracle.c")
LIB = os.path.join(HERE, "libmpqp_oracle.so")

OPTIMAL, UNBOUNDED, ITER_LIMIT, SKIPPED, LICQ_FAIL, INFEASIBLE = range(6)


def build(force: bool = False) -> str:
    """Compile the oracle shared library in place (gcc, no GPU needed)."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                             os.path.getmtime(os.path.join(HERE, "mpqp_oracle.h")))):
        return LIB
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-o", LIB + ".tmp", SRC, "-lm", "-lpthread"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class OrcProblem(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("m", ctypes.c_int), ("p", ctypes.c_int), ("ncp", ctypes.c_int)] + \
        [(nm, ctypes.POINTER(ctypes.c_double)) for nm in ("Q", "c", "H", "A", "b", "F", "At", "bt")]


class OrcTol(ctypes.Structure):
    _fields_ = [("tol_feas", ctypes.c_double), ("tol_opt", ctypes.c_double),
                ("tol_licq", ctypes.c_double), ("r_min", ctypes.c_double),
                ("tol_piv", ctypes.c_double), ("tol_dj", ctypes.c_double),
                ("max_pivots", ctypes.c_int), ("degen_switch", ctypes.c_int), ("tol_zero_row", ctypes.c_double)]


class OrcCand(ctypes.Structure):
    _fields_ = [("mask_lo", ctypes.c_uint64), ("mask_hi", ctypes.c_uint64),
                ("level", ctypes.c_int32), ("parent", ctypes.c_int32),
                ("lp1_status", ctypes.c_int32), ("lp1_pivots", ctypes.c_int32),
                ("z", ctypes.c_double),
                ("feasible", ctypes.c_int32), ("licq", ctypes.c_int32),
                ("optimal", ctypes.c_int32), ("region", ctypes.c_int32),
                ("lp2_status", ctypes.c_int32), ("lp2_pivots", ctypes.c_int32),
                ("cheb_status", ctypes.c_int32), ("cheb_pivots", ctypes.c_int32),
                ("t", ctypes.c_double), ("r", ctypes.c_double)]


CAND_DTYPE = np.dtype([("mask_lo", "<u8"), ("mask_hi", "<u8"), ("level", "<i4"), ("parent", "<i4"),
                       ("lp1_status", "<i4"), ("lp1_pivots", "<i4"), ("z", "<f8"),
                       ("feasible", "<i4"), ("licq", "<i4"), ("optimal", "<i4"), ("region", "<i4"),
                       ("lp2_status", "<i4"), ("lp2_pivots", "<i4"), ("cheb_status", "<i4"),
                       ("cheb_pivots", "<i4"), ("t", "<f8"), ("r", "<f8")])
assert CAND_DTYPE.itemsize == ctypes.sizeof(OrcCand)


class OrcResult(ctypes.Structure):
    _fields_ = [("n_cand", ctypes.c_int64), ("n_pruned", ctypes.c_int64),
                ("n_feasible", ctypes.c_int64), ("n_optimal", ctypes.c_int64),
                ("n_region", ctypes.c_int64), ("n_lp1_pivots", ctypes.c_int64),
                ("n_lp2_pivots", ctypes.c_int64), ("n_cheb_pivots", ctypes.c_int64),
                ("n_levels", ctypes.c_int32), ("truncated", ctypes.c_int32), ("cand", ctypes.POINTER(OrcCand))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.orc_enumerate.argtypes = [ctypes.POINTER(OrcProblem), ctypes.POINTER(OrcTol), ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(OrcResult)]
        _lib.orc_enumerate.restype = ctypes.c_int
        _lib.orc_free_result.argtypes = [ctypes.POINTER(OrcResult)]
        _lib.orc_enumerate_tail.argtypes = [ctypes.POINTER(OrcProblem), ctypes.POINTER(OrcTol), ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(OrcResult)]
        _lib.orc_enumerate_tail.restype = ctypes.c_int
        _lib.orc_check_set.argtypes = [ctypes.POINTER(OrcProblem), ctypes.POINTER(OrcTol),
                                       ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.POINTER(OrcCand),
                                       ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_int)]
        _lib.orc_check_set.restype = ctypes.c_int
        _lib.orc_kkt_data.argtypes = [ctypes.POINTER(OrcProblem)] + [ctypes.POINTER(ctypes.c_double)] * 3
        _lib.orc_kkt_data.restype = ctypes.c_int
        _lib.orc_default_tol.argtypes = [ctypes.POINTER(OrcTol)]
        _lib.orc_lp1_dual_bound.argtypes = [ctypes.POINTER(OrcProblem), ctypes.POINTER(OrcTol),
                                            ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_double,
                                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_int)]
        _lib.orc_lp1_dual_bound.restype = ctypes.c_int
    return _lib


def default_tol(**over) -> OrcTol:
    t = OrcTol()
    lib().orc_default_tol(ctypes.byref(t))
    for k, v in over.items():
        setattr(t, k, v)
    return t


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class _Prob:
    """Keeps the contiguous float64 copies alive for the C structure."""

    def __init__(self, prob):
        self.arrs = [np.ascontiguousarray(getattr(prob, nm), dtype=np.float64)
                     for nm in ("Q", "c", "H", "A", "b", "F", "CRA", "CRb")]
        Q, c, H, A, b, F, CRA, CRb = self.arrs
        self.s = OrcProblem(Q.shape[0], A.shape[0], H.shape[1], CRA.shape[0],
                            *(_dp(a) for a in self.arrs))


@dataclass
class Enumeration:
    n_cand: int
    n_pruned: int
    n_feasible: int
    n_optimal: int
    n_region: int
    n_lp1_pivots: int
    n_lp2_pivots: int
    n_cheb_pivots: int
    n_levels: int
    truncated: int
    cand: np.ndarray | None   # structured array with CAND_DTYPE


def enumerate_sets(prob, k_min: int = 0, k_max: int | None = None, nthreads: int = 1,
                   keep_records: bool = True, tol: OrcTol | None = None, budget: int = 0,
                   exhaustive: bool = False) -> Enumeration:
    pp = _Prob(prob)
    if k_max is None:
        k_max = prob.n
    tol = tol or default_tol()
    res = OrcResult()
    rc = lib().orc_enumerate(ctypes.byref(pp.s), ctypes.byref(tol), k_min, min(k_max, prob.m), int(budget),
                             1 if exhaustive else 0, nthreads, 1 if keep_records else 0, ctypes.byref(res))
    if rc != 0:
        raise RuntimeError(f"oracle enumeration failed: {rc}")
    cand = None
    if keep_records:
        buf = (OrcCand * res.n_cand).from_address(ctypes.addressof(res.cand.contents))
        cand = np.frombuffer(buf, dtype=CAND_DTYPE).copy()
    out = Enumeration(res.n_cand, res.n_pruned, res.n_feasible, res.n_optimal, res.n_region,
                      res.n_lp1_pivots, res.n_lp2_pivots, res.n_cheb_pivots, res.n_levels, res.truncated, cand)
    lib().orc_free_result(ctypes.byref(res))
    return out


def enumerate_tail(prob, j_first: int, k_max: int | None = None, nthreads: int = 1, budget: int = 0,
                   tol: OrcTol | None = None) -> Enumeration:
    """Counts of the enumeration restricted to the sets whose elements are
    all >= j_first (closed under subsets: the same candidates, subset tests,
    warm starts and LPs as the full enumeration, for a bounded sample)."""
    pp = _Prob(prob)
    if k_max is None:
        k_max = prob.n
    tol = tol or default_tol()
    res = OrcResult()
    rc = lib().orc_enumerate_tail(ctypes.byref(pp.s), ctypes.byref(tol), 0, min(k_max, prob.m), int(budget),
                                  nthreads, int(j_first), ctypes.byref(res))
    if rc != 0:
        raise RuntimeError(f"oracle enumeration failed: {rc}")
    out = Enumeration(res.n_cand, res.n_pruned, res.n_feasible, res.n_optimal, res.n_region,
                      res.n_lp1_pivots, res.n_lp2_pivots, res.n_cheb_pivots, res.n_levels, res.truncated, None)
    lib().orc_free_result(ctypes.byref(res))
    return out


def check_set(prob, S, tol: OrcTol | None = None, want_laws: bool = False):
    """Replay the warm-start chain for one sorted active set.

    Returns (record dict, laws dict or None).  laws holds lagrange_A/b,
    parameter_A/b and the normalised region rows CR_As/CR_bs.
    """
    pp = _Prob(prob)
    S = np.ascontiguousarray(sorted(int(s) for s in S), dtype=np.intc)
    k = len(S)
    n, p, m, ncp = prob.n, prob.p, prob.m, prob.ncp
    tol = tol or default_tol()
    rec = OrcCand()
    laws = np.zeros(k * p + k + n * p + n + 1)
    cr = np.zeros(((m + ncp) * (p + 1)) + 1)
    ncr = ctypes.c_int(0)
    rc = lib().orc_check_set(ctypes.byref(pp.s), ctypes.byref(tol),
                             S.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), k, ctypes.byref(rec),
                             _dp(laws) if want_laws else None, _dp(cr) if want_laws else None,
                             ctypes.byref(ncr))
    if rc != 0:
        raise RuntimeError(f"oracle check_set failed: {rc}")
    d = {f[0]: getattr(rec, f[0]) for f in OrcCand._fields_}
    out = None
    if want_laws and d["region"]:
        lA = laws[:k * p].reshape(k, p)
        lb = laws[k * p:k * p + k]
        pA = laws[k * p + k:k * p + k + n * p].reshape(n, p)
        pb = laws[k * p + k + n * p:k * p + k + n * p + n]
        nc = ncr.value
        rows = cr[:nc * (p + 1)].reshape(nc, p + 1)
        out = dict(lagrange_A=lA.copy(), lagrange_b=lb.copy(), parameter_A=pA.copy(),
                   parameter_b=pb.copy(), CR_As=rows[:, :p].copy(), CR_bs=rows[:, p].copy())
    return d, out


def lp1_dual_bound(prob, S, sign_tol: float = 1e-9, tol: OrcTol | None = None):
    """Dual certificate of LP1 infeasibility for a sorted active set.

    Replays the set's warm-start chain up to its first infeasible prefix and
    builds the dual y of that final basis.  Returns (certified, bound, z,
    k_used): certified when y <= c + sign_tol, then bound = beta.y <= z*, the
    LP1 value z of the k_used-element prefix.
    """
    pp = _Prob(prob)
    S = np.ascontiguousarray(sorted(int(s) for s in S), dtype=np.intc)
    tol = tol or default_tol()
    bound, z, used = ctypes.c_double(0.0), ctypes.c_double(0.0), ctypes.c_int(0)
    rc = lib().orc_lp1_dual_bound(ctypes.byref(pp.s), ctypes.byref(tol),
                                  S.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(S), sign_tol,
                                  ctypes.byref(bound), ctypes.byref(z), ctypes.byref(used))
    if rc < 0:
        raise RuntimeError(f"oracle lp1_dual_bound failed: {rc}")
    return rc == 1, bound.value, z.value, used.value


def kkt_data(prob):
    pp = _Prob(prob)
    m, p = prob.m, prob.p
    Wm = np.zeros((m, m)); Wh = np.zeros((m, p)); wc = np.zeros(m)
    rc = lib().orc_kkt_data(ctypes.byref(pp.s), _dp(Wm), _dp(Wh), _dp(wc))
    if rc != 0:
        raise RuntimeError(f"oracle kkt_data failed: {rc}")
    return Wm, Wh, wc


def mask_to_set(lo: int, hi: int) -> list[int]:
    lo, hi = int(lo), int(hi)
    return [j for j in range(64) if lo >> j & 1] + [64 + j for j in range(64) if hi >> j & 1]
