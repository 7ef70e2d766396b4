"""Exact rational dense simplex (fractions.Fraction) — TEST INFRASTRUCTURE ONLY.

A small exact arbiter that travels to any host (glp_exact's library is x86
only).  Textbook two-phase tableau simplex with Bland's rule, so it cannot
cycle; meant for LPs with a few dozen rows.  It follows the same method as
the reference (simplex.cu, tableau from the slack basis, phase I with
artificial columns as simplex.cu:602-826) but in exact arithmetic.

solve(A, b, c) -> (status, objective) with GLPK status codes (5 optimal,
6 unbounded, 4 infeasible) for max c^T x, A x <= b, x >= 0.
"""
from __future__ import annotations

from fractions import Fraction as F


def solve(A, b, c):
    m = len(A)
    n = len(c)
    neg = [i for i in range(m) if b[i] < 0]
    na = len(neg)
    W = n + m + na + 1
    T = [[F(0)] * W for _ in range(m + 1)]
    basis = [0] * m
    k = 0
    for i in range(m):
        s = -1 if b[i] < 0 else 1
        for j in range(n):
            T[i][j] = s * F(A[i][j])
        T[i][n + i] = F(s)
        T[i][W - 1] = s * F(b[i])
        if b[i] < 0:
            T[i][n + m + k] = F(1)
            basis[i] = n + m + k
            k += 1
        else:
            basis[i] = n + i

    def pivot(r, q):
        piv = T[r][q]
        T[r] = [v / piv for v in T[r]]
        for i in range(m + 1):
            if i != r and T[i][q] != 0:
                f = T[i][q]
                T[i] = [a - f * p for a, p in zip(T[i], T[r])]
        basis[r] = q

    def run(ncols):
        while True:
            q = next((j for j in range(ncols) if T[m][j] < 0), -1)
            if q < 0:
                return 5
            best = None
            r = -1
            for i in range(m):
                if T[i][q] > 0:
                    th = T[i][W - 1] / T[i][q]
                    if best is None or th < best or (th == best and basis[i] < basis[r]):
                        best, r = th, i
            if r < 0:
                return 6
            pivot(r, q)

    if na:
        for j in range(W):
            if n + m <= j < W - 1:
                continue
            T[m][j] = -sum((T[i][j] for i in range(m) if basis[i] >= n + m), F(0))
        run(n + m)
        if T[m][W - 1] < 0:
            return 4, None
        for i in range(m):
            if basis[i] >= n + m:
                q = next((j for j in range(n + m) if T[i][j] != 0), -1)
                if q >= 0:
                    pivot(i, q)
        for j in range(W):
            acc = sum((F(c[basis[i]]) * T[i][j] for i in range(m) if basis[i] < n), F(0))
            T[m][j] = acc - (F(c[j]) if j < n else 0)
    else:
        for j in range(n):
            T[m][j] = -F(c[j])
    st = run(n + m)
    return st, T[m][W - 1]


def _solve_int(M, rhs):
    """Exact solve of the square rational system M x = rhs (fraction-free
    Bareiss elimination on an integer-scaled copy).  None if singular."""
    import math
    n = len(M)
    rows = []
    for i in range(n):
        vals = [F(v) for v in M[i]] + [F(rhs[i])]
        den = 1
        for v in vals:
            den = den * v.denominator // math.gcd(den, v.denominator)
        rows.append([v.numerator * (den // v.denominator) for v in vals])
    prev = 1
    for k in range(n):
        p = next((i for i in range(k, n) if rows[i][k] != 0), None)
        if p is None:
            return None
        rows[k], rows[p] = rows[p], rows[k]
        rk = rows[k]
        pk = rk[k]
        for i in range(k + 1, n):
            ri = rows[i]
            f = ri[k]
            if f == 0:
                for j in range(k + 1, n + 1):
                    ri[j] = ri[j] * pk // prev
            else:
                for j in range(k + 1, n + 1):
                    ri[j] = (ri[j] * pk - f * rk[j]) // prev
            ri[k] = 0
        prev = pk
    x = [F(0)] * n
    for i in reversed(range(n)):
        s = F(rows[i][n])
        ri = rows[i]
        for j in range(i + 1, n):
            if ri[j]:
                s -= ri[j] * x[j]
        x[i] = s / ri[i]
    return x


def certify(A, b, c, basic):
    """Exact optimality certificate of a basis for max c^T x, A x <= b, x >= 0.

    `basic` lists m basic column ids (0..n-1 structural, n..n+m-1 slack).
    Solves B x_B = b and B^T y = c_B exactly, then checks x_B >= 0 and every
    reduced cost y^T a_j - c_j >= 0 (slack k: y_k >= 0).  Returns
    (True, objective) when the basis is provably optimal, else (False, None)."""
    m = len(A)
    n = len(c)
    basic = list(basic)
    if len(basic) != m:
        return False, None

    def col(j):
        if j < n:
            return [A[i][j] for i in range(m)]
        return [1 if i == j - n else 0 for i in range(m)]

    cols = [col(j) for j in basic]
    B = [[cols[k][i] for k in range(m)] for i in range(m)]
    BT = [[cols[i][k] for k in range(m)] for i in range(m)]
    cB = [c[j] if j < n else 0 for j in basic]
    xB = _solve_int(B, list(b))
    if xB is None or any(v < 0 for v in xB):
        return False, None
    y = _solve_int(BT, cB)
    if y is None or any(v < 0 for v in y):
        return False, None
    Af = [[F(v) for v in row] for row in A]
    for j in range(n):
        dj = sum((y[i] * Af[i][j] for i in range(m) if Af[i][j] != 0), F(0)) - F(c[j])
        if dj < 0:
            return False, None
    obj = sum((F(cB[k]) * xB[k] for k in range(m)), F(0))
    return True, obj


def unbounded_ray(A, c):
    """A column with every entry <= 0 and a positive cost: x_j can grow
    without bound, so the LP is unbounded (an exact certificate)."""
    m = len(A)
    for j in range(len(c)):
        if c[j] > 0 and all(A[i][j] <= 0 for i in range(m)):
            return True
    return False
