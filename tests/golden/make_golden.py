"""Generates ddla_golden.npz: seeded inputs and the oracle's outputs for the
hot-path operations at sizes that cross DDLA's blocking thresholds
(nb = 128: LU blocked iff n >= 128, Cholesky / LDL^T iff n > 128; GEMM
KC = 144, MR x NR = 6 x 8 edges).

    python tests/golden/make_golden.py      (from the repository root)

The oracle (oracle/ddla_oracle.c) restates DDLA's managed algorithms; these
fixtures freeze its results so that the GPU parity tests and the oracle's own
regression test compare against fixed bytes.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as orc  # noqa: E402

SEED = 0xDD1A0100


def spd(r, n):
    G = r.standard_normal((n, n))
    return G @ G.T / n + np.eye(n)


def sym(L):
    """Symmetric matrix from its stored lower triangle."""
    return L + np.tril(L, -1).T


def main():
    r = np.random.default_rng(SEED)
    out = {}
    # GEMM (config-1 semantics: alpha = 1, beta = 0.5, U[-1,1]) across KC / MR / NR edges
    A, B, C0 = r.uniform(-1, 1, (40, 150)), r.uniform(-1, 1, (150, 50)), r.uniform(-1, 1, (40, 50))
    Cm = C0.copy()
    orc.dgemm(1.0, A, B, 0.5, Cm)
    out.update(gemm_a=A, gemm_b=B, gemm_c0=C0, gemm_c=Cm)
    # GEMMT lower with B = A^T (SYRK shape) and a general B
    A, B, C0 = r.uniform(-1, 1, (60, 150)), r.uniform(-1, 1, (150, 60)), r.uniform(-1, 1, (60, 60))
    Cm = C0.copy()
    orc.dgemmt(orc.LOWER, -1.0, A, B, 1.0, Cm)
    out.update(gemmt_a=A, gemmt_b=B, gemmt_c0=C0, gemmt_c=Cm)
    # TRSM left lower unit (the LU row-block solve)
    T = np.tril(r.uniform(-1, 1, (130, 130)), -1) + np.eye(130)
    B0 = r.uniform(-1, 1, (130, 7))
    X = B0.copy()
    orc.dtrsm(orc.LEFT, orc.LOWER, orc.TRANS_NO, orc.UNIT, 1.0, T, X)
    out.update(trsm_a=np.tril(T), trsm_b=B0, trsm_x=X)
    # PLU, n = 130 (blocked), N(0,1), and its solve
    A = r.standard_normal((130, 130))
    F = A.copy()
    info, piv = orc.dgetrf(F)
    assert info == 0
    b = r.standard_normal((130, 1))
    x = b.copy()
    orc.dgetrs(F, piv, x)
    out.update(plu_a=A, plu_f=F, plu_piv=piv, plu_b=b, plu_x=x)
    # PLU with exact ties between pivot candidates (small integers): first max wins
    A = r.integers(-2, 3, (64, 64)).astype(np.float64) + 5 * np.eye(64)
    F = A.copy()
    info, piv = orc.dgetrf(F)
    out.update(plutie_a=A, plutie_f=F, plutie_piv=piv, plutie_info=np.int32(info))
    # PLU of a singular matrix: LAPACK-style 1-based failing index
    A = r.standard_normal((40, 40))
    A[:, 17] = 0.0
    F = A.copy()
    info, piv = orc.dgetrf(F)
    out.update(plusing_a=A, plusing_info=np.int32(info))
    # LU without pivoting, n = 129, diagonally dominant
    A = r.standard_normal((129, 129)) + 129 * np.eye(129)
    F = A.copy()
    assert orc.dgetrf_nopiv(F) == 0
    out.update(lunp_a=A, lunp_f=F)
    # Cholesky lower / upper, n = 129, 16 right-hand sides
    A = spd(r, 129)
    B0 = r.standard_normal((129, 16))
    for name, uplo in (("lo", orc.LOWER), ("up", orc.UPPER)):
        F = A.copy()
        assert orc.dpotrf(uplo, F) == 0
        X = B0.copy()
        orc.dpotrs(uplo, F, X)
        # only the factor's triangle is meaningful (the other keeps A's values)
        F = np.tril(F) if uplo == orc.LOWER else np.triu(F)
        out.update({f"chol{name}_f": F, f"chol{name}_x": X})
    out.update(chol_a=np.tril(A), chol_b=B0)   # symmetric: the lower triangle is stored
    # Cholesky failure on an indefinite matrix
    A = spd(r, 50)
    A[30, 30] = -1.0
    out.update(cholfail_a=A, cholfail_info=np.int32(orc.dpotrf(orc.LOWER, A.copy())))
    # LDL^T lower, n = 129, and its solve
    A = spd(r, 129)
    F = A.copy()
    assert orc.dldlt(orc.LOWER, F) == 0
    b = r.standard_normal((129, 2))
    x = b.copy()
    orc.dldlts(orc.LOWER, F, x)
    out.update(ldlt_a=np.tril(A), ldlt_f=np.tril(F), ldlt_b=b, ldlt_x=x)
    # einsum (config-5 expressions at small sizes, plus a trace / diagonal mode)
    L, R = r.uniform(-1, 1, (3, 20, 30)), r.uniform(-1, 1, (3, 30, 25))
    Cm = np.zeros((3, 20, 25))
    orc.contract("bik,bkj->bij", 1.0, L, R, Cm)
    out.update(ein1_l=L, ein1_r=R, ein1_c=Cm)
    L, R = r.uniform(-1, 1, (5, 6, 7, 4)), r.uniform(-1, 1, (7, 4, 3, 5))
    Cm = np.zeros((5, 6, 3, 5))
    orc.contract("abcd,cdef->abef", 1.0, L, R, Cm)
    out.update(ein2_l=L, ein2_r=R, ein2_c=Cm)
    L, R = r.uniform(-1, 1, (9, 9, 6)), r.uniform(-1, 1, (6, 8))
    Cm = np.zeros((9, 8))
    orc.contract("iij,jk->ik", 1.0, L, R, Cm)
    out.update(ein3_l=L, ein3_r=R, ein3_c=Cm)
    np.savez_compressed(os.path.join(HERE, "ddla_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "ddla_golden.npz"), len(out), "arrays")
    next_rows()


def next_rows():
    """ddla_golden_next.npz: SYMM, TRMM, TRMM3, SYR2K and Householder QR
    (unblocked n <= 256 and blocked n > 256, DDLA/Factorizations/QR.cs:139-149)."""
    r = np.random.default_rng(SEED + 1)
    out = {}
    A, B, C0 = r.uniform(-1, 1, (70, 70)), r.uniform(-1, 1, (70, 50)), r.uniform(-1, 1, (70, 50))
    Cm = C0.copy()
    orc.dsymm(orc.LEFT, orc.LOWER, 1 / np.pi, A, B, np.e, Cm)
    out.update(symm_a=np.tril(A), symm_b=B, symm_c0=C0, symm_c=Cm)
    A, B = r.uniform(-1, 1, (45, 45)), r.uniform(-1, 1, (60, 45))
    X = B.copy()
    orc.dtrmm(orc.RIGHT, orc.UPPER, orc.TRANS_T, orc.UNIT, 1.2, A, X)
    out.update(trmm_a=np.triu(A, 1), trmm_b=B, trmm_x=X)
    A, Bt, C0 = r.uniform(-1, 1, (50, 50)), r.uniform(-1, 1, (40, 50)), r.uniform(-1, 1, (50, 40))
    Cm = C0.copy()
    orc.dtrmm3(orc.LEFT, orc.LOWER, orc.TRANS_NO, orc.NONUNIT, 1.0, A, Bt, 1.0, Cm, tb=orc.TRANS_T)
    out.update(trmm3_a=np.tril(A), trmm3_bt=Bt, trmm3_c0=C0, trmm3_c=Cm)
    A, B, C0 = r.uniform(-1, 1, (60, 30)), r.uniform(-1, 1, (60, 30)), r.uniform(-1, 1, (60, 60))
    Cm = C0.copy()
    orc.dsyr2k(orc.UPPER, 1 / np.pi, A, B, np.e, Cm)
    out.update(syr2k_a=A, syr2k_b=B, syr2k_c0=C0, syr2k_c=np.triu(Cm))
    for name, (m, n) in (("qr1", (130, 70)), ("qr2", (300, 280))):
        A = r.uniform(-1, 1, (m, n))
        F, T = A.copy(), np.zeros((orc.qr_t_rows(m, n), n))
        orc.dgeqrf(F, T)
        b = r.uniform(-1, 1, (m, 2))
        x = orc.dgeqrs(F, T, b)
        k = min(m, n)
        Tu = np.zeros_like(T)
        for j0 in range(0, k, T.shape[0]):
            bb = min(T.shape[0], k - j0)
            Tu[:bb, j0:j0 + bb] = np.triu(T[:bb, j0:j0 + bb])
        out.update({f"{name}_a": A, f"{name}_f": F, f"{name}_t": Tu, f"{name}_b": b, f"{name}_x": x})
    np.savez_compressed(os.path.join(HERE, "ddla_golden_next.npz"), **out)
    print("wrote", os.path.join(HERE, "ddla_golden_next.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
