"""Seeded inputs and error measures shared by the tests."""
import numpy as np


def rng(seed):
    return np.random.default_rng(seed)


def uniform(r, shape):
    return r.uniform(-1.0, 1.0, shape)


def rel_max(x, ref):
    d = np.max(np.abs(x - ref)) if x.size else 0.0
    s = np.max(np.abs(ref)) if ref.size else 0.0
    return d / s if s > 0 else d


def norms(d):
    """(1-norm, Frobenius, inf-norm) like DDLA's Nrm1 / NrmF / NrmInf."""
    return np.abs(d).sum(axis=0).max(), np.sqrt((d * d).sum()), np.abs(d).sum(axis=1).max()


def apply_piv(B, piv, forward=True):
    B = B.copy()
    idx = range(len(piv)) if forward else range(len(piv) - 1, -1, -1)
    for i in idx:
        p = int(piv[i])
        if p:
            B[[i, i + p]] = B[[i + p, i]]
    return B


def make_lmat(X):
    """Unit lower triangle with the random strictly-lower part (Tests MakeLMat)."""
    return np.tril(X, -1) + np.eye(X.shape[0])


def make_umat(X):
    return np.triu(X)


def spd(r, n):
    """G G^T / n + I with G ~ N(0,1) (the SPD Cholesky workload)."""
    G = r.standard_normal((n, n))
    return G @ G.T / n + np.eye(n)


def pivot_tie_ok(A0, piv_a, piv_b):
    """First differing pivot must be a rounding tie: recompute the column with
    an independent LAPACK-style elimination and check the two candidates'
    magnitudes differ by <= 8 u max|col|."""
    import scipy.linalg as sl
    n = A0.shape[0]
    diff = np.nonzero(np.asarray(piv_a) != np.asarray(piv_b))[0]
    if diff.size == 0:
        return True, -1
    i = int(diff[0])
    # Schur complement column i after i elimination steps with piv_a's rows
    P = apply_piv(A0, piv_a[:i], True) if i else A0.copy()
    lu, _ = sl.lu_factor(P[:, :i]) if i else (None, None)
    if i:
        L11 = np.tril(lu[:i, :i], -1) + np.eye(i)
        U11 = np.triu(lu[:i, :i])
        L21 = np.linalg.solve(U11.T, P[i:, :i].T).T
        col = P[i:, i] - L21 @ np.linalg.solve(L11, P[:i, i])
    else:
        col = P[:, 0]
    a, b = abs(col[piv_a[i]]), abs(col[piv_b[i]])
    return abs(a - b) <= 8 * np.finfo(float).eps * np.abs(col).max(), i


def berr(A, X, B):
    """Relative backward error max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf)."""
    X = X.reshape(X.shape[0], -1)
    B = B.reshape(B.shape[0], -1)
    R = B - A @ X
    an = np.abs(A).sum(axis=1).max()
    return float(np.max(np.abs(R).max(axis=0) / (an * np.abs(X).max(axis=0) + np.abs(B).max(axis=0))))


def schur_pivot_gap(A0, piv_ref, i, p_other):
    """Relative gap between the reference pivot candidate and another one at
    elimination step i: the Schur complement column i after the first i steps
    of piv_ref (FP64, from the row-permuted A0), then
    (|col[piv_ref[i]]| - |col[p_other]|) / max|col|, with row offsets relative
    to row i like the pivots.  A small gap means the two rows were nearly tied,
    so lower-precision rounding can pick either."""
    P = apply_piv(A0, piv_ref[:i], True) if i else A0.copy()
    if i:
        y = np.linalg.solve(P[:i, :i], P[:i, i])
        col = P[i:, i] - P[i:, :i] @ y
    else:
        col = P[:, 0]
    a, b = abs(col[int(piv_ref[i])]), abs(col[int(p_other)])
    return (a - b) / np.abs(col).max()
