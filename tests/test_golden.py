"""The oracle against the committed golden fixtures (tests/golden/ddla_golden.npz,
made by tests/golden/make_golden.py): every output is reproduced bit for bit
from the stored inputs, and the LU pivots agree with LAPACK's (an independent
implementation of the same partial-pivoting rule) where no tie occurs."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "ddla_golden.npz"))


def sym(L):
    return L + np.tril(L, -1).T


def test_gemm_golden(orc, g):
    Cm = g["gemm_c0"].copy()
    orc.dgemm(1.0, g["gemm_a"], g["gemm_b"], 0.5, Cm)
    assert np.array_equal(Cm, g["gemm_c"])
    Cm = g["gemmt_c0"].copy()
    orc.dgemmt(orc.LOWER, -1.0, g["gemmt_a"], g["gemmt_b"], 1.0, Cm)
    assert np.array_equal(Cm, g["gemmt_c"])


def test_trsm_golden(orc, g):
    X = g["trsm_b"].copy()
    orc.dtrsm(orc.LEFT, orc.LOWER, orc.TRANS_NO, orc.UNIT, 1.0, g["trsm_a"] + np.triu(np.ones((130, 130)), 1) * 7,
              X)   # the strict upper triangle must not be read
    assert np.array_equal(X, g["trsm_x"])


def test_plu_golden(orc, g):
    F = g["plu_a"].copy()
    info, piv = orc.dgetrf(F)
    assert info == 0 and np.array_equal(piv, g["plu_piv"]) and np.array_equal(F, g["plu_f"])
    x = g["plu_b"].copy()
    orc.dgetrs(F, piv, x)
    assert np.array_equal(x, g["plu_x"])
    sl = pytest.importorskip("scipy.linalg")
    _, lp = sl.lu_factor(g["plu_a"])
    assert np.array_equal(lp - np.arange(130), g["plu_piv"])   # LAPACK ipiv is absolute


def test_plu_ties_and_singular_golden(orc, g):
    F = g["plutie_a"].copy()
    info, piv = orc.dgetrf(F)
    assert info == int(g["plutie_info"]) and np.array_equal(piv, g["plutie_piv"]) and np.array_equal(F, g["plutie_f"])
    info, _ = orc.dgetrf(g["plusing_a"].copy())
    assert info == int(g["plusing_info"]) > 0


def test_lu_nopiv_golden(orc, g):
    F = g["lunp_a"].copy()
    assert orc.dgetrf_nopiv(F) == 0
    assert np.array_equal(F, g["lunp_f"])


def test_cholesky_golden(orc, g):
    A = sym(g["chol_a"])
    for name, uplo, tri in (("lo", orc.LOWER, np.tril), ("up", orc.UPPER, np.triu)):
        F = A.copy()
        assert orc.dpotrf(uplo, F) == 0
        assert np.array_equal(tri(F), g[f"chol{name}_f"])
        X = g["chol_b"].copy()
        orc.dpotrs(uplo, F, X)
        assert np.array_equal(X, g[f"chol{name}_x"])
    assert orc.dpotrf(orc.LOWER, g["cholfail_a"].copy()) == int(g["cholfail_info"]) == 31


def test_ldlt_golden(orc, g):
    F = sym(g["ldlt_a"])
    assert orc.dldlt(orc.LOWER, F) == 0
    assert np.array_equal(np.tril(F), g["ldlt_f"])
    x = g["ldlt_b"].copy()
    orc.dldlts(orc.LOWER, F, x)
    assert np.array_equal(x, g["ldlt_x"])


@pytest.mark.parametrize("i,expr", [(1, "bik,bkj->bij"), (2, "abcd,cdef->abef"), (3, "iij,jk->ik")])
def test_einsum_golden(orc, g, i, expr):
    Cm = np.zeros_like(g[f"ein{i}_c"])
    orc.contract(expr, 1.0, g[f"ein{i}_l"], g[f"ein{i}_r"], Cm)
    assert np.array_equal(Cm, g[f"ein{i}_c"])
    assert np.allclose(Cm, np.einsum(expr, g[f"ein{i}_l"], g[f"ein{i}_r"]), rtol=0, atol=1e-12)


@pytest.fixture(scope="module")
def gn():
    return np.load(os.path.join(HERE, "golden", "ddla_golden_next.npz"))


def test_level3_next_golden(orc, gn):
    """SYMM / TRMM / TRMM3 / SYR2K: the stored triangles only (the other
    triangle is NaN here, and must not be read)."""
    nan_up = lambda x: x + np.triu(np.full(x.shape, np.nan), 1)      # noqa: E731
    Cm = gn["symm_c0"].copy()
    orc.dsymm(orc.LEFT, orc.LOWER, 1 / np.pi, nan_up(gn["symm_a"]), gn["symm_b"], np.e, Cm)
    assert np.array_equal(Cm, gn["symm_c"])
    A = gn["trmm_a"] + np.tril(np.full((45, 45), np.nan))              # strict upper stored, unit diagonal
    X = gn["trmm_b"].copy()
    orc.dtrmm(orc.RIGHT, orc.UPPER, orc.TRANS_T, orc.UNIT, 1.2, A, X)
    assert np.array_equal(X, gn["trmm_x"])
    Cm = gn["trmm3_c0"].copy()
    orc.dtrmm3(orc.LEFT, orc.LOWER, orc.TRANS_NO, orc.NONUNIT, 1.0, nan_up(gn["trmm3_a"]), gn["trmm3_bt"], 1.0, Cm,
               tb=orc.TRANS_T)
    assert np.array_equal(Cm, gn["trmm3_c"])
    Cm = gn["syr2k_c0"].copy()
    orc.dsyr2k(orc.UPPER, 1 / np.pi, gn["syr2k_a"], gn["syr2k_b"], np.e, Cm)
    assert np.array_equal(np.triu(Cm), gn["syr2k_c"])


@pytest.mark.parametrize("name", ["qr1", "qr2"])
def test_qr_golden(orc, gn, name):
    A = gn[f"{name}_a"]
    m, n = A.shape
    F, T = A.copy(), np.zeros((orc.qr_t_rows(m, n), n))
    orc.dgeqrf(F, T)
    assert np.array_equal(F, gn[f"{name}_f"])
    k = min(m, n)
    for j0 in range(0, k, T.shape[0]):
        b = min(T.shape[0], k - j0)
        assert np.array_equal(np.triu(T[:b, j0:j0 + b]), gn[f"{name}_t"][:b, j0:j0 + b])
    assert np.array_equal(orc.dgeqrs(F, T, gn[f"{name}_b"]), gn[f"{name}_x"])
