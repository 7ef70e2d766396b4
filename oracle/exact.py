"""Exact rational dense simplex (fractions.Fraction) — TEST INFRASTRUCTURE ONLY.

A small exact judge that travels to any host (glp_exact's library is x86
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
