"""The allocation-free region-laws entry point against the allocating one.

``mpqp_region_laws_noalloc`` serves callers that may not allocate device
memory (a control loop past its start-up, or a host that owns the device
memory through its own allocator): they pass host-side problem data and
active sets and device output buffers they allocated themselves.  Here the
output buffers come from torch; the entry point itself allocates nothing.
Two calls in a row, on different problems, must each reproduce the laws of
``mpqp_region_laws`` (the same 1e-12 relative bar as the other law tests),
which also shows that the shared scratch array is fully rewritten per call.
This file is collected last so that a failing run stops after every other
test has run; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 1 << 20


def _bind(lib):
    f = lib.mpqp_region_laws_noalloc
    f.argtypes = [ctypes.POINTER(solver.Problem), ctypes.c_longlong, ctypes.POINTER(ctypes.c_uint64),
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _masks(sets):
    m = np.zeros((len(sets), 2), dtype=np.uint64)
    for i, S in enumerate(sets):
        for j in S:
            m[i, j // 64] |= np.uint64(1) << np.uint64(j % 64)
    return m


def _regions(prob, kmax):
    res = solver.solve([prob], precision=solver.FP64, k_max=kmax, cand_cap=1 << 18, arena_bytes=1 << 28)
    return [solver.mask_to_set(o["mask_lo"], o["mask_hi"]) for o in res.opt if o["region"]]


def _call_noalloc(lib, prob, sets):
    import torch
    f = _bind(lib)
    ps = solver._ProblemSet([prob], 0, 0, 0)
    stride = lib.mpqp_region_laws_stride(ps.arr)
    laws = torch.full((len(sets), stride), float("nan"), dtype=torch.float64, device="cuda")
    sizes = torch.full((len(sets), 4), -7, dtype=torch.int32, device="cuda")
    masks = _masks(sets)
    stream = torch.cuda.current_stream()
    rc = f(ps.arr, len(sets), masks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), laws.data_ptr(),
           sizes.data_ptr(), stream.cuda_stream)
    assert rc == 0, solver.last_error()
    stream.synchronize()
    return laws.cpu().numpy(), sizes.cpu().numpy()


def _check_against_allocating(prob, sets, laws, sizes):
    ref = solver.region_laws(prob, sets)
    m, n, p = prob.m, prob.n, prob.p
    P1 = p + 1
    for i, (S, law) in enumerate(zip(sets, ref)):
        k, nn, pp, ncr = (int(x) for x in sizes[i])
        assert law is not None and k == len(S) and nn == n and pp == p
        lag = laws[i, :k * P1].reshape(k, P1)
        par = laws[i, m * P1:m * P1 + n * P1].reshape(n, P1)
        cr = laws[i, (m + n) * P1:(m + n) * P1 + ncr * P1].reshape(ncr, P1)
        got = dict(lagrange_A=lag[:, :p], lagrange_b=lag[:, p], parameter_A=par[:, :p], parameter_b=par[:, p],
                   CR_As=cr[:, :p], CR_bs=cr[:, p])
        for key, v in got.items():
            want = np.asarray(law[key])
            assert v.shape == want.shape, key
            den = max(float(np.max(np.abs(want))) if want.size else 0.0, 1e-300)
            assert float(np.max(np.abs(v - want))) / den <= 1e-12 if want.size else True, (S, key)


def test_noalloc_matches_allocating_entry_point_two_calls(gpu_lib):
    import torch
    assert torch.cuda.is_available()
    lib = solver.load()
    # first call: the n=4, m=10 problem; second call: a different, larger problem
    p1 = P.scale_problem(P.random_n4_m10_p2())
    s1 = _regions(p1, 4)
    p2 = P.scale_problem(P.random_n12_m62_p6())
    s2 = _regions(p2, 2)[:300]
    assert s1 and s2
    laws1, sizes1 = _call_noalloc(lib, p1, s1)
    laws2, sizes2 = _call_noalloc(lib, p2, s2)
    _check_against_allocating(p1, s1, laws1, sizes1)
    _check_against_allocating(p2, s2, laws2, sizes2)


def test_noalloc_rejects_calls_beyond_the_scratch(gpu_lib):
    import torch
    lib = solver.load()
    f = _bind(lib)
    prob = P.scale_problem(P.random_n4_m10_p2())
    ps = solver._ProblemSet([prob], 0, 0, 0)
    n_sets = SCRATCH_BYTES // 16 + 1          # masks alone exceed the scratch
    masks = np.zeros((n_sets, 2), dtype=np.uint64)
    dummy = torch.empty(1, dtype=torch.float64, device="cuda")
    rc = f(ps.arr, n_sets, masks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), dummy.data_ptr(),
           dummy.data_ptr(), 0)
    assert rc == solver.ECAPACITY
    assert "1 MiB" in solver.last_error()
