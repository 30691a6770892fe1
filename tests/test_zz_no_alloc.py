"""The allocation-free region-laws entry point against the allocating one.

``mpqp_region_laws_noalloc`` serves callers that may not allocate device
memory (a control loop past its start-up, or a host that owns the device
memory through its own allocator): they pass host-side problem data and
active sets and device output buffers they allocated themselves.  Here the
output buffers come from torch; the entry point itself allocates nothing.
Two calls in a row, on different problems, must each reproduce the laws of
``mpqp_region_laws`` (the same 1e-12 relative bar as the other law tests),
which also shows that the shared scratch array is fully rewritten per call;
across those calls neither the device's free memory nor torch's allocator
changes.  An mpLP (Q = 0) instance takes the second precompute branch, with
sets of n and of fewer than n constraints (the latter have no unique law and
report size -2 on both entry points).
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


def _outputs(lib, prob, n_sets):
    """Device output buffers, allocated by the caller before any call."""
    import torch
    ps = solver._ProblemSet([prob], 0, 0, 0)
    stride = lib.mpqp_region_laws_stride(ps.arr)
    laws = torch.full((n_sets, stride), float("nan"), dtype=torch.float64, device="cuda")
    sizes = torch.full((n_sets, 4), -7, dtype=torch.int32, device="cuda")
    return laws, sizes


def _call_noalloc(lib, prob, sets, out):
    import torch
    f = _bind(lib)
    ps = solver._ProblemSet([prob], 0, 0, 0)
    laws, sizes = out
    masks = _masks(sets)
    stream = torch.cuda.current_stream()
    rc = f(ps.arr, len(sets), masks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), laws.data_ptr(),
           sizes.data_ptr(), stream.cuda_stream)
    assert rc == 0, solver.last_error()
    stream.synchronize()


def _check_against_allocating(prob, sets, out):
    laws, sizes = (t.cpu().numpy() for t in out)
    ref = solver.region_laws(prob, sets)
    m, n, p = prob.m, prob.n, prob.p
    P1 = p + 1
    for i, (S, law) in enumerate(zip(sets, ref)):
        k, nn, pp, ncr = (int(x) for x in sizes[i])
        if law is None:
            # no law on either side: the LICQ test failed (-1) or an mpLP set
            # with |S| < n (-2)
            assert k in (-1, -2) and (k == -1 or (not prob.Q.any() and len(S) < n)), (S, k)
            continue
        assert k == len(S) and nn == n and pp == p
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
    o1, o2 = _outputs(lib, p1, len(s1)), _outputs(lib, p2, len(s2))
    _call_noalloc(lib, p1, s1, o1)     # the first call on the device (kernel load, symbol address)
    torch.cuda.synchronize()
    free0, used0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    _call_noalloc(lib, p1, s1, o1)
    _call_noalloc(lib, p2, s2, o2)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0 and torch.cuda.memory_allocated() == used0
    _check_against_allocating(p1, s1, o1)
    _check_against_allocating(p2, s2, o2)


def test_noalloc_mplp_instance(gpu_lib):
    """Q = 0: the mpLP precompute (Wm = A A^T, the multiplier law from A H and
    A c) against the allocating entry point, sets with |S| = n (laws) and
    |S| < n (size -2), two calls in a row."""
    lib = solver.load()
    prob = P.scale_problem(P.random_mplp(4, 13, 3, seed=5))
    res = solver.solve([prob], precision=solver.FP64, k_max=prob.n, cand_cap=1 << 18, arena_bytes=1 << 26)
    full = [solver.mask_to_set(o["mask_lo"], o["mask_hi"]) for o in res.opt if o["level"] == prob.n]
    short = [solver.mask_to_set(o["mask_lo"], o["mask_hi"]) for o in res.opt if o["level"] < prob.n]
    assert full and short
    sets = full[:50] + short[:20]
    for _ in range(2):
        out = _outputs(lib, prob, len(sets))
        _call_noalloc(lib, prob, sets, out)
        _check_against_allocating(prob, sets, out)
        sizes = out[1].cpu().numpy()
        assert all(int(sizes[len(full[:50]) + i, 0]) == -2 for i in range(len(short[:20])))


def test_noalloc_refuses_stream_capture(gpu_lib):
    """A call may not be recorded into a CUDA graph (its upload reads a host
    staging buffer that later calls rewrite): on a capturing stream it
    returns MPQP_EINVAL and enqueues nothing."""
    import torch
    lib = solver.load()
    f = _bind(lib)
    prob = P.scale_problem(P.random_n4_m10_p2())
    sets = _regions(prob, 4)
    out = _outputs(lib, prob, len(sets))
    _call_noalloc(lib, prob, sets, out)
    ps = solver._ProblemSet([prob], 0, 0, 0)
    masks = _masks(sets)
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        g.capture_begin(capture_error_mode="thread_local")
        rc = f(ps.arr, len(sets), masks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), out[0].data_ptr(),
               out[1].data_ptr(), s.cuda_stream)
        g.capture_end()
    assert rc == solver.EINVAL and "captured" in solver.last_error()
    # the next call outside the capture works
    _call_noalloc(lib, prob, sets, out)
    _check_against_allocating(prob, sets, out)


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
