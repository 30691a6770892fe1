"""ctypes front end of libmpqp_gb300.so (the native interface).

The library must have been built in place (``build.py``); there is no CPU
fallback: every entry point here fails loudly when the shared library is
missing or when a CUDA call fails.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

FP64, MIXED = 0, 1
OK, EINVAL, ENOTSPD, EORIGIN, ELAYOUT, ECUDA, ECAPACITY, ENOMEM = 0, -1, -2, -3, -4, -5, -6, -7


class MpqpError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mpqp error {code}: {msg}")
        self.code = code


class Problem(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("m", ctypes.c_int), ("p", ctypes.c_int), ("ncp", ctypes.c_int),
                ("k_min", ctypes.c_int), ("k_max", ctypes.c_int), ("budget", ctypes.c_longlong)] + \
        [(nm, ctypes.POINTER(ctypes.c_double)) for nm in ("Q", "c", "H", "A", "b", "F", "At", "bt")]


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("exhaustive", ctypes.c_int), ("record", ctypes.c_int),
                ("use_graph", ctypes.c_int), ("cand_cap", ctypes.c_longlong), ("node_cap", ctypes.c_longlong),
                ("arena_bytes", ctypes.c_longlong), ("rec_cap", ctypes.c_longlong), ("opt_cap", ctypes.c_longlong),
                ("mem_fraction", ctypes.c_double),
                ("tol_feas", ctypes.c_double), ("tol_opt", ctypes.c_double), ("tol_licq", ctypes.c_double),
                ("r_min", ctypes.c_double), ("tol_piv", ctypes.c_double), ("tol_dj", ctypes.c_double),
                ("max_pivots", ctypes.c_int), ("degen_switch", ctypes.c_int),
                ("tol_piv32", ctypes.c_double), ("tol_dj32", ctypes.c_double), ("margin_z", ctypes.c_double),
                ("margin_beta", ctypes.c_double), ("margin_t", ctypes.c_double), ("margin_licq", ctypes.c_double),
                ("tol_zero_row", ctypes.c_double), ("lp2_screen", ctypes.c_int),
                ("tile_w", ctypes.c_int), ("feas_warps", ctypes.c_int), ("feas_chunk", ctypes.c_int),
                ("autotune", ctypes.c_int), ("lp2_warm", ctypes.c_int)]


class OptSet(ctypes.Structure):
    _fields_ = [("mask_lo", ctypes.c_uint64), ("mask_hi", ctypes.c_uint64), ("inst", ctypes.c_int),
                ("level", ctypes.c_int), ("t", ctypes.c_double), ("r", ctypes.c_double), ("region", ctypes.c_int),
                ("fp64", ctypes.c_int), ("rec", ctypes.c_longlong), ("err", ctypes.c_double)]


class InstStats(ctypes.Structure):
    _fields_ = [(nm, ctypes.c_longlong) for nm in ("candidates", "pruned", "feasible", "optimal", "regions",
                                                    "lp1_pivots", "lp2_pivots", "cheb_pivots", "fallback_lp1",
                                                    "fallback_opt", "stored")] + \
        [(nm, ctypes.c_ulonglong) for nm in ("feasible_digest", "optimal_digest", "region_digest")] + \
        [("last_level", ctypes.c_int), ("truncated", ctypes.c_int)] + \
        [(nm, ctypes.c_longlong) for nm in ("lp1_certified", "lp1_cert_missed", "lp1_cert_freevar", "lp1_parents",
                                            "lp1_parent_bytes", "lp1_store_bytes", "lp1_cold",
                                            "nodes_without_tableau", "lp2_first_stage_lps",
                                            "lp2_first_stage_pivots", "lp2_warm_offered", "lp2_warm_started",
                                            "lp2_certified", "lp1_vertex_checked")]


class BatchResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("n_inst", ctypes.c_int), ("n_levels", ctypes.c_int),
                ("overflow", ctypes.c_int), ("device_ms", ctypes.c_double),
                ("inst", ctypes.POINTER(InstStats)), ("n_opt", ctypes.c_longlong), ("opt", ctypes.POINTER(OptSet)),
                ("n_rec", ctypes.c_longlong), ("rec", ctypes.c_void_p), ("h2d_bytes", ctypes.c_longlong),
                ("d2h_bytes", ctypes.c_longlong), ("tile_w", ctypes.c_int), ("feas_warps", ctypes.c_int),
                ("feas_chunk", ctypes.c_int), ("tuned", ctypes.c_int), ("split_levels", ctypes.c_int),
                ("pad_", ctypes.c_int)]


class GPUResults(ctypes.Structure):
    """The reference's result structure (main.py:12-22) plus appended fields."""
    _fields_ = [('n_batches', ctypes.c_int), ('n_splits', ctypes.c_int), ('n_feasible_lps', ctypes.c_int),
                ('n_final_lps', ctypes.c_int), ('time_feas', ctypes.c_double), ('time_opti', ctypes.c_double),
                ('time_GPU', ctypes.c_double), ('active_sets', ctypes.POINTER(ctypes.c_int)),
                ('status', ctypes.c_int), ('n_regions', ctypes.c_int), ('n_candidates', ctypes.c_longlong),
                ('n_pruned', ctypes.c_longlong), ('t_star', ctypes.POINTER(ctypes.c_double)),
                ('radius', ctypes.POINTER(ctypes.c_double)), ('is_region', ctypes.POINTER(ctypes.c_int)),
                ('law_error', ctypes.POINTER(ctypes.c_double))]


# record layout written by the device (identical prefix to the oracle's)
REC_DTYPE = np.dtype([("mask_lo", "<u8"), ("mask_hi", "<u8"), ("level", "<i4"), ("parent", "<i4"),
                      ("lp1_status", "<i4"), ("lp1_pivots", "<i4"), ("z", "<f8"),
                      ("feasible", "<i4"), ("licq", "<i4"), ("optimal", "<i4"), ("region", "<i4"),
                      ("lp2_status", "<i4"), ("lp2_pivots", "<i4"), ("cheb_status", "<i4"),
                      ("cheb_pivots", "<i4"), ("t", "<f8"), ("r", "<f8"), ("inst", "<i4"), ("fp64", "<i4"),
                      ("lp1_growth", "<f4"), ("lp1_minbeta", "<f4"), ("lp1_bound", "<f8")])

EXPORTS = ("mpqp", "warm_up", "mpqp_free", "mpqp_unpack_lp", "mpqp_default_options", "mpqp_solve_batch", "mpqp_batch_free",
           "mpqp_plan_create", "mpqp_plan_run", "mpqp_plan_results", "mpqp_plan_launches", "mpqp_plan_destroy",
           "mpqp_plan_run_timed", "mpqp_plan_kernel_times",
           "mpqp_region_laws_stride", "mpqp_region_laws", "mpqp_critical_regions", "mpqp_reduce_constraints",
           "mpqp_release_cached_memory", "mpqp_region_laws_noalloc",
           "mpqp_version",
           "mpqp_last_error")

_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the in-tree shared library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(f"libmpqp_gb300.so not built ({path}); run mpqpcudasolver_gb300.build.build()")
    lib = ctypes.CDLL(path)
    P, PP = ctypes.POINTER, ctypes.POINTER(ctypes.POINTER(BatchResult))
    lib.mpqp.argtypes = [P(ctypes.c_double), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                         ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_int), ctypes.c_int,
                         ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_int), P(ctypes.c_int),
                         ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.mpqp.restype = P(GPUResults)
    lib.mpqp_free.argtypes = [P(GPUResults)]
    dp = P(ctypes.c_double)
    lib.mpqp_unpack_lp.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_int, ctypes.c_int,
                                   dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int] + [dp] * 8 + [P(ctypes.c_int)]
    lib.mpqp_unpack_lp.restype = ctypes.c_int
    lib.mpqp_default_options.argtypes = [P(Options)]
    lib.mpqp_solve_batch.argtypes = [ctypes.c_int, P(Problem), P(Options), PP]
    lib.mpqp_solve_batch.restype = ctypes.c_int
    lib.mpqp_batch_free.argtypes = [P(BatchResult)]
    lib.mpqp_plan_create.argtypes = [ctypes.c_int, P(Problem), P(Options), P(ctypes.c_void_p)]
    lib.mpqp_plan_create.restype = ctypes.c_int
    lib.mpqp_plan_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.mpqp_plan_run.restype = ctypes.c_int
    lib.mpqp_plan_results.argtypes = [ctypes.c_void_p, PP]
    lib.mpqp_plan_results.restype = ctypes.c_int
    lib.mpqp_plan_launches.argtypes = [ctypes.c_void_p]
    lib.mpqp_plan_launches.restype = ctypes.c_int
    lib.mpqp_plan_destroy.argtypes = [ctypes.c_void_p]
    lib.mpqp_plan_run_timed.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.mpqp_plan_run_timed.restype = ctypes.c_int
    lib.mpqp_plan_kernel_times.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, P(ctypes.c_double),
                                           P(ctypes.c_int)]
    lib.mpqp_plan_kernel_times.restype = ctypes.c_int
    lib.mpqp_region_laws_stride.argtypes = [P(Problem)]
    lib.mpqp_region_laws_stride.restype = ctypes.c_longlong
    lib.mpqp_region_laws.argtypes = [P(Problem), ctypes.c_longlong, P(ctypes.c_uint64), P(ctypes.c_double),
                                     P(ctypes.c_int)]
    lib.mpqp_region_laws.restype = ctypes.c_int
    lib.mpqp_critical_regions.argtypes = [P(Problem), ctypes.c_longlong, P(ctypes.c_uint64), P(ctypes.c_double),
                                          P(ctypes.c_int), P(ctypes.c_double), P(ctypes.c_double)]
    lib.mpqp_critical_regions.restype = ctypes.c_int
    lib.mpqp_reduce_constraints.argtypes = [P(Problem), P(ctypes.c_int)]
    lib.mpqp_reduce_constraints.restype = ctypes.c_int
    lib.mpqp_release_cached_memory.restype = ctypes.c_int
    lib.mpqp_version.restype = ctypes.c_char_p
    lib.mpqp_last_error.restype = ctypes.c_char_p
    _lib = lib
    return lib


def last_error() -> str:
    return load().mpqp_last_error().decode()


def _check(rc: int):
    if rc != 0:
        raise MpqpError(rc, last_error())


def default_options(**over) -> Options:
    o = Options()
    load().mpqp_default_options(ctypes.byref(o))
    for k, v in over.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


class _ProblemSet:
    """Contiguous float64 copies kept alive for the C structures."""

    def __init__(self, probs, k_min=0, k_max=None, budget=0):
        self.keep = []
        self.arr = (Problem * len(probs))()
        for i, pr in enumerate(probs):
            arrs = [np.ascontiguousarray(getattr(pr, nm), dtype=np.float64)
                    for nm in ("Q", "c", "H", "A", "b", "F", "CRA", "CRb")]
            self.keep.append(arrs)
            kmax = pr.n if k_max is None else (k_max[i] if isinstance(k_max, (list, tuple)) else k_max)
            bud = budget[i] if isinstance(budget, (list, tuple)) else budget
            s = self.arr[i]
            s.n, s.m, s.p, s.ncp = pr.n, pr.m, pr.p, pr.CRA.shape[0]
            s.k_min, s.k_max, s.budget = k_min, min(kmax, pr.m), int(bud)
            for nm, a in zip(("Q", "c", "H", "A", "b", "F", "At", "bt"), arrs):
                setattr(s, nm, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))


@dataclass
class Result:
    status: int
    device_ms: float
    n_levels: int
    overflow: int
    inst: np.ndarray          # structured per-instance counters
    opt: np.ndarray           # structured optimal sets
    rec: np.ndarray | None    # structured records (record=1)
    h2d_bytes: int = 0
    d2h_bytes: int = 0
    settings: dict | None = None   # launch settings of the run (tile_w, feas_warps, feas_chunk, tuned)
    split_levels: int = 0          # levels whose feasible sets did not all keep an LP1 tableau

    @property
    def candidates(self) -> int:
        return int(self.inst["candidates"].sum())

    def total(self, field: str) -> int:
        return int(self.inst[field].sum())


_INST_DTYPE = np.dtype([(f[0], "<i8") for f in InstStats._fields_[:11]] +
                       [("feasible_digest", "<u8"), ("optimal_digest", "<u8"), ("region_digest", "<u8"),
                        ("last_level", "<i4"), ("truncated", "<i4"), ("lp1_certified", "<i8"),
                        ("lp1_cert_missed", "<i8"), ("lp1_cert_freevar", "<i8"), ("lp1_parents", "<i8"),
                        ("lp1_parent_bytes", "<i8"), ("lp1_store_bytes", "<i8"), ("lp1_cold", "<i8"),
                        ("nodes_without_tableau", "<i8"), ("lp2_first_stage_lps", "<i8"),
                        ("lp2_first_stage_pivots", "<i8"), ("lp2_warm_offered", "<i8"),
                        ("lp2_warm_started", "<i8"), ("lp2_certified", "<i8"), ("lp1_vertex_checked", "<i8")])
_OPT_DTYPE = np.dtype([("mask_lo", "<u8"), ("mask_hi", "<u8"), ("inst", "<i4"), ("level", "<i4"), ("t", "<f8"),
                       ("r", "<f8"), ("region", "<i4"), ("fp64", "<i4"), ("rec", "<i8"), ("err", "<f8")])
assert _INST_DTYPE.itemsize == ctypes.sizeof(InstStats)
assert _OPT_DTYPE.itemsize == ctypes.sizeof(OptSet)


def _convert(rp) -> Result:
    r = rp.contents
    ni = r.n_inst
    inst = np.frombuffer((InstStats * ni).from_address(ctypes.addressof(r.inst.contents)), dtype=_INST_DTYPE).copy()
    nopt = r.n_opt
    opt = (np.frombuffer((OptSet * nopt).from_address(ctypes.addressof(r.opt.contents)), dtype=_OPT_DTYPE).copy()
           if nopt else np.zeros(0, dtype=_OPT_DTYPE))
    rec = None
    if r.rec:
        nrec = r.n_rec
        buf = (ctypes.c_char * (nrec * REC_DTYPE.itemsize)).from_address(r.rec)
        rec = np.frombuffer(buf, dtype=REC_DTYPE).copy()
    settings = dict(tile_w=r.tile_w, feas_warps=r.feas_warps, feas_chunk=r.feas_chunk, tuned=r.tuned)
    return Result(r.status, r.device_ms, r.n_levels, r.overflow, inst, opt, rec, r.h2d_bytes, r.d2h_bytes, settings,
                  r.split_levels)


def solve(probs, precision: int = FP64, k_min: int = 0, k_max=None, budget=0, **opts) -> Result:
    """Run the whole enumeration for a list of MPQP instances in one launch sequence."""
    lib = load()
    ps = _ProblemSet(probs, k_min, k_max, budget)
    o = default_options(precision=precision, **opts)
    out = ctypes.POINTER(BatchResult)()
    rc = lib.mpqp_solve_batch(len(probs), ps.arr, ctypes.byref(o), ctypes.byref(out))
    if not out:
        _check(rc if rc else ECUDA)
    res = _convert(out)
    lib.mpqp_batch_free(out)
    _check(rc)
    return res


class Plan:
    """Device-resident problem set: upload once, run many times."""

    def __init__(self, probs, precision: int = FP64, k_min: int = 0, k_max=None, budget=0, **opts):
        self.lib = load()
        self.ps = _ProblemSet(probs, k_min, k_max, budget)
        self.opts = default_options(precision=precision, **opts)
        self.h = ctypes.c_void_p()
        _check(self.lib.mpqp_plan_create(len(probs), self.ps.arr, ctypes.byref(self.opts), ctypes.byref(self.h)))

    def run(self, stream: int = 0):
        _check(self.lib.mpqp_plan_run(self.h, ctypes.c_void_p(stream)))

    def results(self) -> Result:
        out = ctypes.POINTER(BatchResult)()
        rc = self.lib.mpqp_plan_results(self.h, ctypes.byref(out))
        if not out:
            _check(rc if rc else ECUDA)
        res = _convert(out)
        self.lib.mpqp_batch_free(out)
        _check(rc)
        return res

    def run_timed(self, stream: int = 0):
        """One run without the graph, with a CUDA event around every launch."""
        _check(self.lib.mpqp_plan_run_timed(self.h, ctypes.c_void_p(stream)))

    def kernel_times(self) -> dict:
        """{kernel name: (total ms, launches)} of the last timed run."""
        nmax = 32
        names = ctypes.create_string_buffer(64 * nmax)
        ms = (ctypes.c_double * nmax)()
        cnt = (ctypes.c_int * nmax)()
        n = self.lib.mpqp_plan_kernel_times(self.h, nmax, names, ms, cnt)
        if n < 0:
            _check(n)
        return {names.raw[64 * i:64 * i + 64].split(b"\0")[0].decode(): (ms[i], cnt[i]) for i in range(n)}

    @property
    def launches(self) -> int:
        return self.lib.mpqp_plan_launches(self.h)

    def close(self):
        if self.h:
            self.lib.mpqp_plan_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# row status codes of mpqp_reduce_constraints
ROW_KEPT, ROW_ZERO, ROW_DUPLICATE, ROW_EQUALITY_PAIR, ROW_REDUNDANT, ROW_EQUALITY = range(6)


def reduce_constraints(prob):
    """Constraint reduction on the device (zero, duplicate, implicit-equality
    and redundant rows; the ppopt steps of utils.py:163-190).

    Returns (status, reduced): ``status`` holds one code per row of A, then
    per row of CRA; ``reduced`` is a copy of ``prob`` with the removed rows
    dropped (row order kept) and ``meta["kept_rows"]`` / ``meta["kept_param_rows"]``
    / ``meta["equality_rows"]`` (indices into the reduced A) recorded."""
    lib = load()
    ps = _ProblemSet([prob], 0, 0, 0)
    status = np.zeros(prob.m + prob.ncp, dtype=np.intc)
    _check(lib.mpqp_reduce_constraints(ps.arr, status.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
    return status, apply_row_status(prob, status)


def apply_row_status(prob, status):
    """The problem with the rows that ``status`` marks as removed dropped.

    Rows of the parameter set (CRA) found redundant are kept: active sets
    index rows of A only, a redundant row changes no critical region, and the
    LP layout of the reference's call (main.py:91-98) needs at least one
    parameter row (the box can be implied by the rows of A, which would leave
    none).  Zero and duplicate parameter rows are dropped."""
    m = prob.m
    keep = [i for i in range(m) if status[i] in (ROW_KEPT, ROW_EQUALITY)]
    keep_t = [i for i in range(prob.ncp) if status[m + i] in (ROW_KEPT, ROW_EQUALITY, ROW_REDUNDANT)]
    out = prob.copy()
    out.A, out.b, out.F = prob.A[keep], prob.b[keep], prob.F[keep]
    out.CRA, out.CRb = prob.CRA[keep_t], prob.CRb[keep_t]
    for name in ("A", "b", "F", "CRA", "CRb"):
        setattr(out, name, np.ascontiguousarray(getattr(out, name), dtype=np.float64))
    out.meta = dict(prob.meta, kept_rows=keep, kept_param_rows=keep_t,
                    equality_rows=[j for j, i in enumerate(keep) if status[i] == ROW_EQUALITY])
    return out


def region_laws(prob, sets, with_radius: bool = False):
    """FP64 laws of the given active sets (device).  Returns a list of dicts;
    None for a set that fails the LICQ test and for an mpLP set with fewer
    than n active constraints (its law x(theta) is not unique).  with_radius:
    each dict also holds the set's Chebyshev radius ``r`` (``mpqp_critical_regions``;
    a critical region when r >= 1e-8, utils.py:86) and the stated relative
    error ``err`` of its laws (one FP64 iterative-refinement step)."""
    lib = load()
    ps = _ProblemSet([prob], 0, 0, 0)
    masks = np.zeros((len(sets), 2), dtype=np.uint64)
    for i, S in enumerate(sets):
        for j in S:
            masks[i, j // 64] |= np.uint64(1) << np.uint64(j % 64)
    stride = lib.mpqp_region_laws_stride(ps.arr)
    laws = np.zeros((max(len(sets), 1), stride))
    sizes = np.zeros((max(len(sets), 1), 4), dtype=np.intc)
    radius = np.full(max(len(sets), 1), np.nan)
    err = np.full(max(len(sets), 1), np.nan)
    args = (ps.arr, len(sets), masks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            laws.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    if with_radius:
        _check(lib.mpqp_critical_regions(*args, radius.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                         err.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    else:
        _check(lib.mpqp_region_laws(*args))
    out = []
    m, n, p = prob.m, prob.n, prob.p
    P1 = p + 1
    for i in range(len(sets)):
        k, _, _, ncr = sizes[i]
        if k < 0:
            out.append(None)
            continue
        lag = laws[i, :k * P1].reshape(k, P1)
        par = laws[i, m * P1:m * P1 + n * P1].reshape(n, P1)
        cr = laws[i, (m + n) * P1:(m + n) * P1 + ncr * P1].reshape(ncr, P1)
        d = dict(lagrange_A=lag[:, :p].copy(), lagrange_b=lag[:, p].copy(), parameter_A=par[:, :p].copy(),
                 parameter_b=par[:, p].copy(), CR_As=cr[:, :p].copy(), CR_bs=cr[:, p].copy(),
                 active_set=list(sets[i]))
        if with_radius:
            d["r"] = float(radius[i])
            d["err"] = float(err[i])
        out.append(d)
    return out


def unpack_lp(d: dict):
    """Problem arrays that ``mpqp()`` reads back from the LP matrices of
    ``host.build_lp_data`` (host only, no GPU work)."""
    lib = load()
    n_c, n_x, n_t, M1 = d["num_c"], d["num_x"], d["num_t"], d["M1"]
    n_cp = M1 - n_c
    out = {k: np.zeros(sz) for k, sz in (("Q", (n_x, n_x)), ("c", n_x), ("H", (n_x, n_t)), ("A", (n_c, n_x)),
                                           ("b", n_c), ("F", (n_c, n_t)), ("At", (n_cp, n_t)), ("bt", n_cp))}
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    ncp = ctypes.c_int(0)
    rc = lib.mpqp_unpack_lp(dp(d["A0"]), n_c, n_x, n_t, dp(d["A1"]), dp(d["xb1"]), d["M1"], d["N1"], dp(d["A2"]),
                            dp(d["xb2"]), d["M2"], d["N2"], d["n_eqs"], *(dp(out[k]) for k in
                                                                        ("Q", "c", "H", "A", "b", "F", "At", "bt")),
                            ctypes.byref(ncp))
    _check(rc)
    return out


def mask_digest(lo, hi) -> int:
    """The 64-bit hash the device sums into the set digests."""
    M = (1 << 64) - 1

    def mix(x):
        x ^= x >> 33
        x = (x * 0xff51afd7ed558ccd) & M
        x ^= x >> 33
        x = (x * 0xc4ceb9fe1a85ec53) & M
        x ^= x >> 33
        return x
    return mix((int(lo) ^ mix((int(hi) ^ 0x5bd1e9955bd1e995) & M)) & M)


def mask_to_set(lo, hi) -> list[int]:
    lo, hi = int(lo), int(hi)
    return [j for j in range(64) if lo >> j & 1] + [64 + j for j in range(64) if hi >> j & 1]
