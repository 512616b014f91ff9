"""Oracle (test infrastructure only): numpy restatement of the reference's
MMA update, src/MEXfuncs/MMA_mex.cpp:6-54 with the solver class of
src/MEXfuncs/MMAseq.cpp (Svanberg's method of moving asymptotes, sequential
form with a dual interior-point subproblem solver, as written by N. Aage).

MMA_mex builds a fresh MMAseq(n, m, a=0, c=100, d=0) on every call, so its
iteration counter is 1 and the asymptotes are always the initial ones
(MMAseq.cpp:460-466): L = x - 0.5 (xmax - xmin), U = x + 0.5 (xmax - xmin).
The returned xold1 is the incoming x, xold2 the incoming xold1.
"""
from __future__ import annotations

import numpy as np


def mma_update(m, n, xval, xmin, xmax, xold1, xold2, df0dx, fval, dfdx):
    """Returns (xnew, xold1_out, xold2_out).  dfdx: m*n values in the order
    MMA_mex receives them (dfdx_MMA(:), i.e. dgdx[i*m + j])."""
    m, n = int(m), int(n)
    x = np.asarray(xval, float).copy()
    xmin = np.asarray(xmin, float)
    xmax = np.asarray(xmax, float)
    df0 = np.asarray(df0dx, float)
    g = np.atleast_1d(np.asarray(fval, float))
    dg = np.asarray(dfdx, float).reshape(n, m)
    a = np.zeros(m)
    c = np.full(m, 100.0)
    asyminit = 0.5
    # GenSub (MMAseq.cpp:455-545), k = 1
    L = x - asyminit * (xmax - xmin)
    U = x + asyminit * (xmax - xmin)
    feps = 1.0e-6
    alpha = np.maximum(xmin, 0.9 * L + 0.1 * x)
    beta = np.minimum(xmax, 0.9 * U + 0.1 * x)
    p0 = (U - x) ** 2 * (np.maximum(0.0, df0) + 0.001 * np.abs(df0) + 0.5 * feps / (U - L))
    q0 = (x - L) ** 2 * (np.maximum(0.0, -df0) + 0.001 * np.abs(df0) + 0.5 * feps / (U - L))
    pij = (U - x)[:, None] ** 2 * np.maximum(0.0, dg)
    qij = (x - L)[:, None] ** 2 * np.maximum(0.0, -dg)
    b = -g + (pij / (U - x)[:, None] + qij / (x - L)[:, None]).sum(axis=0)
    xo1_out = x.copy()
    xo2_out = np.asarray(xold1, float).copy()

    # SolveDIP (MMAseq.cpp:191-245)
    lam = c / 2.0
    mu = np.ones(m)
    tol = 1.0e-9 * np.sqrt(m + n)
    epsi = 1.0
    err = 1.0

    def xyz(lam):
        lam = np.maximum(lam, 0.0)
        y = np.maximum(0.0, lam - c)
        z = max(0.0, 10.0 * (float(lam @ a) - 1.0))
        pl = p0 + pij @ lam
        ql = q0 + qij @ lam
        xp = (np.sqrt(pl) * L + np.sqrt(ql) * U) / (np.sqrt(pl) + np.sqrt(ql))
        return lam, y, z, np.clip(xp, alpha, beta), xp, pl, ql

    def sums(xx):
        return (pij / (U - xx)[:, None] + qij / (xx - L)[:, None]).sum(axis=0)

    while epsi > tol:
        loop = 0
        while err > 0.9 * epsi and loop < 100:
            loop += 1
            lam, y, z, x, xp, pl, ql = xyz(lam)
            grad = -b - a * z - y + sums(x)
            grad = -grad - epsi / lam
            # DualHess
            PQ = pij / ((U - x) ** 2)[:, None] - qij / ((x - L) ** 2)[:, None]
            df2 = -1.0 / (2.0 * pl / (U - x) ** 3 + 2.0 * ql / (x - L) ** 3)
            df2[(xp < alpha) | (xp > beta)] = 0.0
            H = (PQ * df2[:, None]).T @ PQ
            lam = np.maximum(lam, 0.0)
            lamai = float(lam @ a)
            H[np.diag_indices(m)] += np.where(lam > c, -1.0, 0.0)
            H[np.diag_indices(m)] += -mu / lam
            if lamai > 0.0:
                H += -10.0 * np.outer(a, a)
            corr = 1e-4 * np.trace(H) / m
            if -corr < 1.0e-7:
                corr = -1.0e-7
            H[np.diag_indices(m)] += corr
            s0 = np.linalg.solve(H, grad) if m > 1 else grad / H[0, 0]
            s1 = -mu + epsi / lam - s0 * mu / lam
            # DualLineSearch
            theta = 1.005
            for i in range(m):
                theta = max(theta, -1.01 * s0[i] / lam[i])
                theta = max(theta, -1.01 * s1[i] / mu[i])
            theta = 1.0 / theta
            lam = lam + theta * s0
            mu = mu + theta * s1
            lam, y, z, x, xp, pl, ql = xyz(lam)
            res = np.concatenate([-b - a * z - y + mu + sums(x), mu * lam - epsi])
            err = float(np.abs(res).max())
        epsi *= 0.1
    return x, xo1_out, xo2_out
