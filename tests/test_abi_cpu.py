"""The C-ABI library on the CPU: it builds, loads, exports every symbol the
public header declares, rebuilds the problem from the reference's LP
matrices exactly (host-only entry point), and rejects bad arguments before
any device work; nothing here launches a kernel."""
import ctypes
import os
import re

import numpy as np
import pytest

from mpqpcudasolver_gb300 import build as B
from mpqpcudasolver_gb300 import host
from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "mpqp_gb300.h")


@pytest.fixture(scope="module")
def lib():
    B.build()
    return solver.load()


def header_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = set(re.findall(r"\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", txt))
    return sorted(n for n in names if n not in {"if", "while", "sizeof"})


def test_header_declares_the_reference_entry_points():
    fns = header_functions()
    assert "mpqp" in fns and "warm_up" in fns
    assert len(fns) >= 15


def test_library_exports_every_declared_symbol(lib):
    for name in header_functions():
        assert hasattr(lib, name), name
    for name in solver.EXPORTS:
        assert hasattr(lib, name), name
    assert lib.mpqp_version().startswith(b"mpqp_gb300")


def test_gpu_results_prefix_matches_reference_layout():
    # main.py:12-22: four ints, three doubles, one pointer
    class Ref(ctypes.Structure):
        _fields_ = [('n_batches', ctypes.c_int), ('n_splits', ctypes.c_int), ('n_feasible_lps', ctypes.c_int),
                    ('n_final_lps', ctypes.c_int), ('time_feas', ctypes.c_double), ('time_opti', ctypes.c_double),
                    ('time_GPU', ctypes.c_double), ('active_sets', ctypes.POINTER(ctypes.c_int))]
    for f, _ in Ref._fields_:
        assert getattr(Ref, f).offset == getattr(solver.GPUResults, f).offset, f


@pytest.mark.parametrize("make", [P.random_n4_m10_p2, P.random_n10_m43_p4, P.illcond_n16_m62_p8, lambda: P.mpc_mpqp(3),
                                  lambda: P.batch_member(5), lambda: P.random_mplp(4, 13, 3, seed=5),
                                  lambda: P.random_mplp(6, 20, 3, seed=3, h_scale=0.0)])
def test_unpack_lp_recovers_the_problem(lib, make):
    prog = host.MPQPProb.from_mpqp(make())
    prog.process_constraints(scale_method=1)
    d = host.build_lp_data(prog)
    out = solver.unpack_lp(d)
    assert np.array_equal(out["A"], prog.A)
    assert np.array_equal(out["F"], prog.F)
    assert np.array_equal(out["b"], prog.b.ravel())
    assert np.array_equal(out["At"], prog.A_t)
    assert np.array_equal(out["bt"], prog.b_t.ravel())
    assert np.array_equal(out["Q"], prog.Q)
    assert np.array_equal(out["H"], prog.H)
    assert np.array_equal(out["c"], prog.c.ravel())


def test_unpack_lp_rejects_other_layouts(lib):
    prog = host.MPQPProb.from_mpqp(P.random_n4_m10_p2())
    prog.process_constraints(scale_method=1)
    d = host.build_lp_data(prog)
    bad = dict(d, N1=d["N1"] + 1)
    with pytest.raises(solver.MpqpError) as e:
        solver.unpack_lp(bad)
    assert e.value.code == solver.ELAYOUT
    bad = dict(d, A0=np.asfortranarray(d["A0"] + 1.0))
    with pytest.raises(solver.MpqpError) as e:
        solver.unpack_lp(bad)
    assert e.value.code == solver.ELAYOUT
    # a stationarity row whose multiplier block is not A^T (main.py:106)
    A2 = np.array(d["A2"], order="F", copy=True)
    r0 = d["num_c"] + 1 + (d["M1"] - d["num_c"])
    A2[r0, d["num_x"] + d["num_t"]] += 0.5
    with pytest.raises(solver.MpqpError) as e:
        solver.unpack_lp(dict(d, A2=A2))
    assert e.value.code == solver.ELAYOUT


def test_entry_points_reject_bad_arguments_before_any_device_work(lib):
    """Null plans, empty instance lists and bad options come back as MPQP_EINVAL
    with a message (no CUDA call is reached); the free functions take NULL."""
    out = ctypes.POINTER(solver.BatchResult)()
    assert lib.mpqp_plan_results(None, ctypes.byref(out)) == solver.EINVAL and not out
    assert "not run" in solver.last_error()
    assert lib.mpqp_plan_run(None, None) == solver.EINVAL
    assert lib.mpqp_plan_run_timed(None, None) == solver.EINVAL
    names = ctypes.create_string_buffer(64)
    ms, cnt = (ctypes.c_double * 1)(), (ctypes.c_int * 1)()
    assert lib.mpqp_plan_kernel_times(None, 1, names, ms, cnt) == solver.EINVAL
    assert lib.mpqp_plan_launches(None) == 0
    lib.mpqp_plan_destroy(None)
    lib.mpqp_batch_free(None)
    lib.mpqp_free(None)
    h = ctypes.c_void_p()
    assert lib.mpqp_plan_create(0, None, None, ctypes.byref(h)) == solver.EINVAL and not h.value
    assert "no instances" in solver.last_error()
    assert lib.mpqp_solve_batch(0, None, None, ctypes.byref(out)) == solver.EINVAL and not out
    ps = solver._ProblemSet([P.scale_problem(P.random_n4_m10_p2())])
    opts = solver.Options()
    lib.mpqp_default_options(ctypes.byref(opts))
    assert opts.precision == solver.FP64 and opts.use_graph == 1
    opts.lp2_screen = 7
    assert lib.mpqp_plan_create(1, ps.arr, ctypes.byref(opts), ctypes.byref(h)) == solver.EINVAL and not h.value
    assert "lp2_screen" in solver.last_error()
    opts.lp2_screen = 0
    opts.lp2_warm = 3
    assert lib.mpqp_plan_create(1, ps.arr, ctypes.byref(opts), ctypes.byref(h)) == solver.EINVAL and not h.value
    assert "lp2_warm" in solver.last_error()
    assert lib.mpqp_region_laws(None, 1, None, None, None) == solver.EINVAL
    assert lib.mpqp_region_laws(ps.arr, -1, None, None, None) == solver.EINVAL
    assert lib.mpqp_region_laws(ps.arr, 0, None, None, None) == solver.OK      # nothing to do
    assert lib.mpqp_reduce_constraints(None, None) == solver.EINVAL
    assert lib.mpqp_version().decode().startswith("mpqp_gb300")
