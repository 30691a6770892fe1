"""Seeded synthetic mpQP generators for the benchmark and test workloads.

Every problem has the form used throughout the reference (``main.py:71-80``,
``utils.py:147-161``)::

    min_x  1/2 x^T Q x + (c + H theta)^T x
    s.t.   A x <= b + F theta,      CRA theta <= CRb

There is no public dataset for this metric, so seeded generators with the
stated shapes and distributions stand in for one.  All random draws come from
``numpy.random.default_rng(seed)`` in the order documented in each function,
so a seed fixes the problem bit for bit on every machine.

Workloads (n = #variables, m = #constraints, p = #parameters):

* ``random_n4_m10_p2``    n=4,  m=10, p=2, seed 0 -- small enough for
  exhaustive checks (386 active sets with |S| <= 4).
* ``random_n10_m43_p4``   n=10, m=43, p=4.
* ``m62_batch``           ``random_n12_m62_p6`` (n=12, m=62, p=6) plus 32
  ``batch_member`` instances (seeds 1..32) with n~U{5..15}, m~U{20..80},
  p~U{2..6}: the benchmark batch.
* ``illcond_n16_m62_p8``  n=16, m=62, p=8, Q = U diag(lambda) U^T with U
  Haar-random and lambda log-uniform in [1e-2, 1e2]; 20 % of the constraint
  rows duplicate other rows up to N(0, 1e-12) noise on A, F and b.
* ``mpc_batch``           64 condensed linear-MPC problems (seeds 0..63),
  horizon 6: n=12, m=72, p=4.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class MPQP:
    """One multiparametric QP.  Arrays are float64, C-contiguous.

    ``b`` and ``CRb`` are 1-D.  ``name`` documents the generator and seed.
    """

    Q: np.ndarray
    c: np.ndarray
    H: np.ndarray
    A: np.ndarray
    b: np.ndarray
    F: np.ndarray
    CRA: np.ndarray
    CRb: np.ndarray
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.Q.shape[0]

    @property
    def m(self) -> int:
        return self.A.shape[0]

    @property
    def p(self) -> int:
        return self.H.shape[1]

    @property
    def ncp(self) -> int:
        return self.CRA.shape[0]

    def copy(self) -> "MPQP":
        return MPQP(*(np.array(a, dtype=np.float64, copy=True) for a in
                      (self.Q, self.c, self.H, self.A, self.b, self.F, self.CRA, self.CRb)),
                    name=self.name, meta=dict(self.meta))


def _box(p: int, half_width: float):
    CRA = np.vstack([np.eye(p), -np.eye(p)])
    CRb = np.full(2 * p, float(half_width))
    return CRA, CRb


def random_mpqp(n: int, m: int, p: int, seed: int, box: float = 1.0,
                rng: np.random.Generator | None = None) -> MPQP:
    """Plain random mpQP (the generator of every ``random_*`` workload).

    Draw order: M (n x n) N(0,1); c N(0,1); H (n x p) N(0,1); A (m x n) N(0,1)
    with unit-norm rows; b U[1,2] (so the origin is strictly feasible);
    F (m x p) N(0, 0.25), 0.25 read as the variance (std 0.5).
    Q = M M^T + I.  theta box [-box, box]^p.
    """
    if rng is None:
        rng = np.random.default_rng(seed)
    M = rng.standard_normal((n, n))
    c = rng.standard_normal(n)
    H = rng.standard_normal((n, p))
    A = rng.standard_normal((m, n))
    A /= np.linalg.norm(A, axis=1, keepdims=True)
    b = rng.uniform(1.0, 2.0, m)
    F = rng.normal(0.0, 0.5, (m, p))
    Q = M @ M.T + np.eye(n)
    CRA, CRb = _box(p, box)
    return MPQP(Q, c, H, A, b, F, CRA, CRb, name=f"random(n={n},m={m},p={p},seed={seed})")


def random_mplp(n: int, m: int, p: int, seed: int, box: float = 1.0, h_scale: float = 1.0) -> MPLP:
    """Random multiparametric LP (Q = 0), bounded for every theta.

    Draw order: c N(0,1); H (n x p) N(0,1) times ``h_scale`` (the cost
    (c + H theta)^T x moves with theta; 0 gives a fixed cost); A0
    ((m - 2n) x n) N(0,1) with unit-norm rows; b U[1,2] (m); F0
    ((m - 2n) x p) N(0, 0.25), 0.25 read as the variance.  A = [A0; I; -I]
    (the last 2n rows bound x), F = [F0; 0], theta box [-box, box]^p.
    """
    if m < 2 * n + 1:
        raise ValueError("random_mplp needs m >= 2n + 1")
    rng = np.random.default_rng(seed)
    c = rng.standard_normal(n)
    H = rng.standard_normal((n, p)) * h_scale
    A0 = rng.standard_normal((m - 2 * n, n))
    A0 /= np.linalg.norm(A0, axis=1, keepdims=True)
    b = rng.uniform(1.0, 2.0, m)
    F0 = rng.normal(0.0, 0.5, (m - 2 * n, p))
    A = np.vstack([A0, np.eye(n), -np.eye(n)])
    F = np.vstack([F0, np.zeros((2 * n, p))])
    CRA, CRb = _box(p, box)
    return MPQP(np.zeros((n, n)), c, H, np.ascontiguousarray(A), b, np.ascontiguousarray(F), CRA, CRb,
                name=f"random_mplp(n={n},m={m},p={p},seed={seed},h_scale={h_scale})")


MPLP = MPQP   # an mpLP is an MPQP whose Q is zero


def random_n4_m10_p2() -> MPQP:
    return random_mpqp(4, 10, 2, seed=0)


def random_n10_m43_p4() -> MPQP:
    return random_mpqp(10, 43, 4, seed=0)


def random_n12_m62_p6() -> MPQP:
    return random_mpqp(12, 62, 6, seed=0)


def batch_member(seed: int) -> MPQP:
    """One extra instance of the m = 62 batch; its sizes are drawn first from
    the same stream (n~U{5..15}, m~U{20..80}, p~U{2..6})."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(5, 16))
    m = int(rng.integers(20, 81))
    p = int(rng.integers(2, 7))
    prob = random_mpqp(n, m, p, seed=seed, rng=rng)
    prob.name = f"batch_member(seed={seed},n={n},m={m},p={p})"
    return prob


def m62_batch(n_extra: int = 32) -> list[MPQP]:
    return [random_n12_m62_p6()] + [batch_member(s) for s in range(1, n_extra + 1)]


def illcond_n16_m62_p8(seed: int = 0) -> MPQP:
    """Ill-conditioned Q and near-duplicate constraint rows.

    Draw order: Gaussian G (n x n) -> U = QR(G) with the sign fix
    U *= sign(diag(R)); log10(lambda) U[-2, 2]; c; H; A (unit rows); b U[1,2];
    F N(0, 0.25); then the duplicate map and the three noise blocks.
    20 % of the rows (round(0.2 m)) are replaced by a copy of a different,
    non-duplicated row; A, F and b of the copy each receive N(0, 1e-12) noise
    (1e-12 read as the standard deviation).  b of the copy is copied too.
    """
    n, m, p = 16, 62, 8
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((n, n))
    U, R = np.linalg.qr(G)
    U = U * np.sign(np.diag(R))[None, :]
    lam = 10.0 ** rng.uniform(-2.0, 2.0, n)
    Q = (U * lam[None, :]) @ U.T
    Q = 0.5 * (Q + Q.T)
    c = rng.standard_normal(n)
    H = rng.standard_normal((n, p))
    A = rng.standard_normal((m, n))
    A /= np.linalg.norm(A, axis=1, keepdims=True)
    b = rng.uniform(1.0, 2.0, m)
    F = rng.normal(0.0, 0.5, (m, p))
    n_dup = int(round(0.2 * m))
    dup_rows = rng.choice(m, size=n_dup, replace=False)
    originals = np.setdiff1d(np.arange(m), dup_rows)
    src = rng.choice(originals, size=n_dup, replace=True)
    A[dup_rows] = A[src] + rng.normal(0.0, 1e-12, (n_dup, n))
    F[dup_rows] = F[src] + rng.normal(0.0, 1e-12, (n_dup, p))
    b[dup_rows] = b[src] + rng.normal(0.0, 1e-12, n_dup)
    CRA, CRb = _box(p, 1.0)
    return MPQP(Q, c, H, A, b, F, CRA, CRb, name=f"illcond_n16_m62_p8(seed={seed})",
                meta={"dup_rows": dup_rows.tolist(), "dup_src": src.tolist()})


def mpc_mpqp(seed: int, horizon: int = 6) -> MPQP:
    """Condensed linear MPC as an mpQP in the initial state theta = x0.

    Draw order: A_d (4x4) N(0,1) rescaled to spectral radius 0.95; B_d (4x2)
    N(0,1).  Q_x = I, R = 0.1 I, terminal P from the discrete algebraic
    Riccati equation.  Decision vector U = (u_0..u_{N-1}) (n = 2N = 12).
    Constraints |u_k| <= 1 (24 rows) and |x_k| <= 5 for k = 1..N (48 rows),
    theta in [-3, 3]^4.
    """
    from scipy.linalg import solve_discrete_are

    rng = np.random.default_rng(seed)
    nx, nu, N = 4, 2, horizon
    Ad = rng.standard_normal((nx, nx))
    rho = np.max(np.abs(np.linalg.eigvals(Ad)))
    Ad = Ad * (0.95 / rho)
    Bd = rng.standard_normal((nx, nu))
    Qx = np.eye(nx)
    Ru = 0.1 * np.eye(nu)
    P = solve_discrete_are(Ad, Bd, Qx, Ru)
    P = 0.5 * (P + P.T)
    # x_k = Ad^k x0 + sum_{j<k} Ad^{k-1-j} Bd u_j  for k = 1..N
    Sx = np.zeros((N * nx, nx))
    Su = np.zeros((N * nx, N * nu))
    Ak = np.eye(nx)
    for k in range(1, N + 1):
        Ak = Ad @ Ak
        Sx[(k - 1) * nx:k * nx] = Ak
        for j in range(k):
            Su[(k - 1) * nx:k * nx, j * nu:(j + 1) * nu] = np.linalg.matrix_power(Ad, k - 1 - j) @ Bd
    Qbar = np.zeros((N * nx, N * nx))
    for k in range(N - 1):
        Qbar[k * nx:(k + 1) * nx, k * nx:(k + 1) * nx] = Qx
    Qbar[(N - 1) * nx:, (N - 1) * nx:] = P
    Rbar = np.kron(np.eye(N), Ru)
    Q = 2.0 * (Su.T @ Qbar @ Su + Rbar)
    Q = 0.5 * (Q + Q.T)
    H = 2.0 * (Su.T @ Qbar @ Sx)
    c = np.zeros(N * nu)
    A = np.vstack([np.eye(N * nu), -np.eye(N * nu), Su, -Su])
    b = np.concatenate([np.ones(2 * N * nu), np.full(2 * N * nx, 5.0)])
    F = np.vstack([np.zeros((2 * N * nu, nx)), -Sx, Sx])
    CRA, CRb = _box(nx, 3.0)
    return MPQP(Q, c, H, A, b, F, CRA, CRb, name=f"mpc(seed={seed})")


def mpc_batch(n_instances: int = 64) -> list[MPQP]:
    return [mpc_mpqp(s) for s in range(n_instances)]


def scale_problem(prob: MPQP) -> MPQP:
    """The numerical preprocessing the reference applies before its C call.

    Restates ``MPQPProb.process_constraints(scale_method=1)``
    (``utils.py:163-199``) without its ppopt steps (zero/duplicate/redundant
    row removal and implicit-equality detection, ``utils.py:165-190``), which
    are outside the accelerated path:

    * ``scale_AF`` (``utils.py:208-221``): each row of [A F] and b is divided
      by max|[A F]| of that row (rows of zeros keep scale 1);
    * ``scale_At`` (``utils.py:223-229``): the same for CRA / CRb;
    * Q, H, c are divided by max|[Q H c]| / 8 (``utils.py:193-199``).
    """
    out = prob.copy()
    AF = np.hstack([out.A, out.F])
    R = np.max(np.abs(AF), axis=1)
    R[R == 0] = 1
    R = 1 / R
    out.A = out.A * R.reshape(-1, 1)
    out.F = out.F * R.reshape(-1, 1)
    out.b = out.b * R
    Rt = np.max(np.abs(out.CRA), axis=1)
    Rt[Rt == 0] = 1
    Rt = 1 / Rt
    out.CRA = out.CRA * Rt.reshape(-1, 1)
    out.CRb = out.CRb * Rt
    QHc = np.hstack([out.Q, out.H, out.c.reshape(-1, 1)])
    norm = np.max(np.abs(QHc)) / (2 ** 3)
    out.Q = out.Q / norm
    out.H = out.H / norm
    out.c = out.c / norm
    for name in ("Q", "c", "H", "A", "b", "F", "CRA", "CRb"):
        setattr(out, name, np.ascontiguousarray(getattr(out, name), dtype=np.float64))
    return out


def mplp_member(seed: int) -> MPQP:
    """One instance of the mpLP batch; sizes drawn first from the same stream
    (n ~ U{4..8}, m ~ U{2n+6..2n+16}, p ~ U{2..4}), then ``random_mplp``
    with a parametric cost (h_scale 1) on that stream."""
    rng = np.random.default_rng(10_000 + seed)
    n = int(rng.integers(4, 9))
    m = int(rng.integers(2 * n + 6, 2 * n + 17))
    p = int(rng.integers(2, 5))
    prob = random_mplp(n, m, p, seed=10_000 + seed)
    prob.name = f"mplp_member(seed={seed},n={n},m={m},p={p})"
    return prob


def mplp_batch(n_instances: int = 32) -> list[MPQP]:
    """32 random mpLPs (Q = 0) of mixed sizes, enumerated to |S| = n."""
    return [mplp_member(s) for s in range(n_instances)]


def pop_like_set(n_problems: int = 24, seed: int = 0, n_max: int = 5, m_max: int = 16) -> list[MPQP]:
    """A seeded stand-in for a set of test problems of mixed sizes (the
    reference's driver loops over a public test set, which is not copied
    here).  Problem i: sizes drawn from ``default_rng(seed)`` in the order
    n ~ U{2..n_max}, m ~ U{n+2..m_max}, p ~ U{2..4}, box ~ U[1, 3]; then
    ``random_mpqp(n, m, p, seed=seed*1000+i, box)``."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_problems):
        n = int(rng.integers(2, n_max + 1))
        m = int(rng.integers(n + 2, m_max + 1))
        p = int(rng.integers(2, 5))
        box = float(rng.uniform(1.0, 3.0))
        prob = random_mpqp(n, m, p, seed=seed * 1000 + i, box=box)
        prob.name = f"pop_like(seed={seed},i={i},n={n},m={m},p={p})"
        out.append(prob)
    return out


WORKLOADS = {
    "n4-m10-p2": lambda: [random_n4_m10_p2()],
    "n10-m43-p4": lambda: [random_n10_m43_p4()],
    "m62-batch": m62_batch,
    "n12-m62-p6": lambda: [random_n12_m62_p6()],
    "illcond-n16-m62-p8": lambda: [illcond_n16_m62_p8()],
    "mpc-batch": mpc_batch,
    "pop-like": pop_like_set,
    "mplp-batch": mplp_batch,
}
