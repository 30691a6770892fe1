"""Exact rational verdicts for small problems (test infrastructure only).

Every float64 input is converted exactly to a ``fractions.Fraction``; LP1,
the KKT solve and LP2 then run in exact arithmetic with Bland's rule, so the
verdicts carry no rounding at all:

* feasible  <=>  min sum_{i in S} w_i == 0 over [A -F; 0 At] u + w = [b; bt],
  w >= 0, u free (the LP1 of main.py:91-98 / batched_simplex.cu:26-36,308-314);
* LICQ      <=>  A_S Q^-1 A_S^T is nonsingular;
* optimal   <=>  max t > 0 over {lambda_S(theta) >= t, inactive slacks >= t,
  At theta <= bt} (the LP2 of main.py:102-128 after eliminating x, lambda).

The Chebyshev radius needs square roots, so the region verdict is pinned
through its exact equivalent: a region of positive radius exists iff t* > 0.
"""
from __future__ import annotations

from fractions import Fraction
from itertools import combinations


def _F(x) -> Fraction:
    return Fraction(float(x))


def _inv(M):
    """Exact inverse by Gauss-Jordan (raises on singular)."""
    n = len(M)
    A = [row[:] + [Fraction(int(i == j)) for j in range(n)] for i, row in enumerate(M)]
    for c in range(n):
        piv = next((r for r in range(c, n) if A[r][c] != 0), None)
        if piv is None:
            raise ZeroDivisionError("singular")
        A[c], A[piv] = A[piv], A[c]
        pv = A[c][c]
        A[c] = [v / pv for v in A[c]]
        for r in range(n):
            if r != c and A[r][c] != 0:
                f = A[r][c]
                A[r] = [a - f * b for a, b in zip(A[r], A[c])]
    return [row[n:] for row in A]


def _tucker(T, bid, nid, nfree):
    """Bland's-rule Tucker simplex, minimising the last row; returns status."""
    nrows = len(T) - 1
    ncols = len(T[0]) - 1
    while True:
        obj = T[nrows]
        q = None
        for j in sorted(range(ncols), key=lambda j: nid[j]):
            g = obj[j]
            if (nid[j] < nfree and g != 0) or g > 0:
                q = j
                break
        if q is None:
            return "optimal"
        sg = 1 if obj[q] > 0 else -1
        r, best = None, None
        for i in range(nrows):
            if bid[i] < nfree:
                continue
            a = sg * T[i][q]
            if a > 0:
                ratio = max(T[i][ncols], Fraction(0)) / a
                if best is None or ratio < best or (ratio == best and bid[i] < bid[r]):
                    r, best = i, ratio
        if r is None:
            return "unbounded"
        inv = 1 / T[r][q]
        T[r] = [v * inv if j != q else inv for j, v in enumerate(T[r])]
        for i in range(nrows + 1):
            if i == r:
                continue
            f = T[i][q]
            if f != 0:
                T[i] = [T[i][j] - f * T[r][j] if j != q else -f * inv for j in range(ncols + 1)]
        bid[r], nid[q] = nid[q], bid[r]


class ExactProblem:
    def __init__(self, prob):
        self.n, self.m, self.p, self.ncp = prob.n, prob.m, prob.p, prob.CRA.shape[0]
        n, m, p = self.n, self.m, self.p
        self.Q = [[_F(v) for v in row] for row in prob.Q]
        self.c = [_F(v) for v in prob.c]
        self.H = [[_F(v) for v in row] for row in prob.H]
        self.A = [[_F(v) for v in row] for row in prob.A]
        self.b = [_F(v) for v in prob.b]
        self.F = [[_F(v) for v in row] for row in prob.F]
        self.At = [[_F(v) for v in row] for row in prob.CRA]
        self.bt = [_F(v) for v in prob.CRb]
        Qi = _inv(self.Q)
        QiAT = [[sum(Qi[r][k] * self.A[i][k] for k in range(n)) for i in range(m)] for r in range(n)]
        self.Wm = [[sum(self.A[i][k] * QiAT[k][j] for k in range(n)) for j in range(m)] for i in range(m)]
        QiH = [[sum(Qi[r][k] * self.H[k][c] for k in range(n)) for c in range(p)] for r in range(n)]
        Qic = [sum(Qi[r][k] * self.c[k] for k in range(n)) for r in range(n)]
        self.Wh = [[sum(self.A[i][k] * QiH[k][c] for k in range(n)) + self.F[i][c] for c in range(p)]
                   for i in range(m)]
        self.wc = [sum(self.A[i][k] * Qic[k] for k in range(n)) + self.b[i] for i in range(m)]

    def lp1_value(self, S) -> Fraction:
        n, m, p, ncp = self.n, self.m, self.p, self.ncp
        nv = n + p
        rows = [self.A[i] + [-v for v in self.F[i]] + [self.b[i]] for i in range(m)]
        rows += [[Fraction(0)] * n + self.At[i] + [self.bt[i]] for i in range(ncp)]
        obj = [sum((rows[i][j] for i in S), Fraction(0)) for j in range(nv + 1)]
        T = [r[:] for r in rows] + [obj]
        bid = [nv + i for i in range(m + ncp)]
        nid = list(range(nv))
        st = _tucker(T, bid, nid, nv)
        assert st == "optimal"
        return T[-1][nv]

    def lp2_value(self, S):
        """(licq, t*) with t* = None when LP2 is infeasible."""
        m, p = self.m, self.p
        S = list(S)
        k = len(S)
        if k:
            try:
                Mi = _inv([[self.Wm[a][b] for b in S] for a in S])
            except ZeroDivisionError:
                return False, None
            B = [self.Wh[s] + [self.wc[s]] for s in S]
            Lam = [[sum(Mi[a][l] * B[l][c] for l in range(k)) for c in range(p + 1)] for a in range(k)]
        else:
            Lam = []
        G = []
        for a in range(k):
            G.append(Lam[a][:p] + [-Lam[a][p]])
        Sset = set(S)
        for i in range(m):
            if i in Sset:
                continue
            g = [sum((self.Wm[i][S[l]] * Lam[l][c] for l in range(k)), Fraction(0)) - self.Wh[i][c]
                 for c in range(p)]
            h = self.wc[i] - sum((self.Wm[i][S[l]] * Lam[l][p] for l in range(k)), Fraction(0))
            G.append(g + [h])
        t0 = min(r[p] for r in G)
        T = [r[:p] + [Fraction(1), r[p] - t0] for r in G]
        T += [self.At[i] + [Fraction(0), self.bt[i]] for i in range(self.ncp)]
        T.append([Fraction(0)] * p + [Fraction(1), -t0])
        bid = [p + 1 + r for r in range(len(T) - 1)]
        nid = list(range(p + 1))
        st = _tucker(T, bid, nid, p + 1)
        if st == "unbounded":
            return True, None
        t = -T[-1][p + 1]
        return True, t

    def verdict(self, S):
        z = self.lp1_value(S)
        feasible = z == 0
        licq, t, optimal = None, None, False
        if feasible:
            licq, t = self.lp2_value(S)
            optimal = bool(licq and t is not None and t > 0)
        return dict(feasible=feasible, z=z, licq=licq, t=t, optimal=optimal)


def exhaustive_verdicts(prob, k_max: int):
    """Exact verdicts of every active set with |S| <= k_max."""
    E = ExactProblem(prob)
    out = {}
    for k in range(k_max + 1):
        for S in combinations(range(E.m), k):
            out[S] = E.verdict(S)
    return out
