"""Host-side logic on the CPU: generators, preprocessing, result decoding and
the multi-rank aggregation of bench.py (two gloo ranks)."""
import os
import sys

import numpy as np
import pytest

from mpqpcudasolver_gb300 import host
from mpqpcudasolver_gb300 import problems as P
from oracle import reference_lp as R

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_generators_are_deterministic_and_shaped():
    a, b = P.random_n4_m10_p2(), P.random_n4_m10_p2()
    for k in ("Q", "c", "H", "A", "b", "F", "CRA", "CRb"):
        assert np.array_equal(getattr(a, k), getattr(b, k))
    assert (a.n, a.m, a.p) == (4, 10, 2)
    assert np.allclose(np.linalg.norm(a.A, axis=1), 1.0)
    assert a.b.min() >= 1.0 and a.b.max() <= 2.0
    c3 = P.m62_batch(n_extra=32)
    assert len(c3) == 33 and (c3[0].n, c3[0].m, c3[0].p) == (12, 62, 6)
    for pr in c3[1:]:
        assert 5 <= pr.n <= 15 and 20 <= pr.m <= 80 and 2 <= pr.p <= 6
    c4 = P.illcond_n16_m62_p8()
    assert (c4.n, c4.m, c4.p) == (16, 62, 8)
    ev = np.linalg.eigvalsh(c4.Q)
    assert ev.min() > 0 and 5e3 < ev.max() / ev.min() < 1e4 + 1
    d, s = np.array(c4.meta["dup_rows"]), np.array(c4.meta["dup_src"])
    assert len(d) == round(0.2 * c4.m)
    assert np.max(np.abs(c4.A[d] - c4.A[s])) < 1e-10 and np.max(np.abs(c4.b[d] - c4.b[s])) < 1e-10
    m5 = P.mpc_mpqp(7)
    assert (m5.n, m5.m, m5.p) == (12, 72, 4)
    assert np.allclose(m5.CRb, 3.0)


def test_scaling_restates_the_reference_and_is_idempotent():
    raw = P.random_n10_m43_p4()
    s1 = P.scale_problem(raw)
    assert np.allclose(np.max(np.abs(np.hstack([s1.A, s1.F])), axis=1), 1.0)
    assert np.isclose(np.max(np.abs(np.hstack([s1.Q, s1.H, s1.c[:, None]]))), 8.0)
    s2 = P.scale_problem(s1)
    for k in ("Q", "c", "H", "A", "b", "F", "CRA", "CRb"):
        assert np.allclose(getattr(s1, k), getattr(s2, k), rtol=1e-15, atol=0)


def test_lp_builders_agree():
    prog = host.MPQPProb.from_mpqp(P.random_n10_m43_p4())
    prog.process_constraints(scale_method=1)
    d = host.build_lp_data(prog)
    r = R.build_lp_matrices(prog.to_mpqp())
    for k in ("A1", "A2", "b1", "b2", "non_b2"):
        assert np.array_equal(d[k], r[k]), k
    assert np.array_equal(d["xb1"], r["xb1"]) and np.array_equal(d["xb2"], r["xb2"])


def test_decode_active_sets():
    rows = np.array([0, 3, -1, -1, 2, -1, -1, -1, 1, 2, 3, 4], dtype=np.intc)
    assert host.decode_active_sets(rows, 3, 4) == [[0, 3], [2], [1, 2, 3, 4]]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [100.0, 250.0][rank]
    worst = bench.max_over_ranks(ms, dist, device="cpu")
    q.put((rank, worst, bench.whole_job_rate(1000, worst, world)))
    dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank_over_gloo():
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, worst, rate in res:
        assert worst == 250.0
        assert rate == pytest.approx(2 * 1000 / 0.25)
