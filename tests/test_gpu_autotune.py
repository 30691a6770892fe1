"""The launch-setting autotuner.

The reference takes its threads per LP from host code (the launch shapes of
batched_simplex.cu:1181 and around).  Here three settings are chosen per
batch shape: threads per LP in the first stage of the FP32 screen (8, 16 or
32: 4, 2 or 1 LPs per warp), warps per LP1 block and candidates an LP1 warp
claims at a time.  Every setting must give the same verdicts (checked against
the FP64 path over the whole grid of settings); the tuner must pick settings
from that grid, record them in the result, and reuse its choice for the next
plan of the same shape.
"""
import itertools

import numpy as np
import pytest

from mpqpcudasolver_gb300 import problems as P
from mpqpcudasolver_gb300 import solver

pytestmark = pytest.mark.gpu

FIELDS = ("candidates", "feasible", "optimal", "regions", "feasible_digest", "optimal_digest", "region_digest")


def _batch():
    probs = [P.scale_problem(P.random_n12_m62_p6()), P.scale_problem(P.random_n10_m43_p4()),
             P.scale_problem(P.mpc_mpqp(1)), P.scale_problem(P.illcond_n16_m62_p8())]
    return probs, [3, 4, 3, 3]


def test_every_setting_gives_the_same_verdicts(gpu_lib):
    probs, kmax = _batch()
    kw = dict(k_max=kmax, cand_cap=1 << 21, arena_bytes=1 << 29)
    ref = solver.solve(probs, precision=solver.FP64, **kw)
    assert ref.status == 0
    for tw, fw, fc in itertools.product((8, 16, 32), (1, 2, 4), (1, 8, 32)):
        r = solver.solve(probs, precision=solver.MIXED, tile_w=tw, feas_warps=fw, feas_chunk=fc, **kw)
        assert r.status == 0
        assert r.settings == dict(tile_w=tw, feas_warps=fw, feas_chunk=fc, tuned=0)
        for f in FIELDS:
            assert np.array_equal(r.inst[f], ref.inst[f]), (tw, fw, fc, f)
    # the FP64 path's LP1 takes the same settings
    for fw, fc in ((1, 1), (2, 16)):
        r = solver.solve(probs, precision=solver.FP64, feas_warps=fw, feas_chunk=fc, **kw)
        for f in FIELDS:
            assert np.array_equal(r.inst[f], ref.inst[f]), (fw, fc, f)


def test_tuner_picks_and_records_a_valid_setting(gpu_lib):
    probs, kmax = _batch()
    kw = dict(k_max=kmax, cand_cap=1 << 21, arena_bytes=1 << 29)
    ref = solver.solve(probs, precision=solver.FP64, **kw)
    a = solver.solve(probs, precision=solver.MIXED, autotune=1, **kw)
    s = a.settings
    assert s["tuned"] == 1 and s["tile_w"] in (8, 16, 32)
    assert (s["feas_warps"], s["feas_chunk"]) in ((4, 32), (4, 16), (2, 32), (4, 8), (2, 16))
    for f in FIELDS:
        assert np.array_equal(a.inst[f], ref.inst[f]), f
    # the same shape again: the cached choice
    b = solver.solve(probs, precision=solver.MIXED, autotune=1, **kw)
    assert b.settings == s
    # an explicit setting is kept, the others tuned
    c = solver.solve(probs, precision=solver.MIXED, autotune=1, tile_w=32, **kw)
    assert c.settings["tile_w"] == 32 and c.settings["tuned"] == 1
    print("tuned settings", s)


def test_bad_settings_are_rejected(gpu_lib):
    probs, kmax = _batch()
    for bad in (dict(tile_w=4), dict(feas_warps=5), dict(feas_chunk=33)):
        with pytest.raises(solver.MpqpError):
            solver.solve(probs[:1], precision=solver.MIXED, k_max=1, **bad)
