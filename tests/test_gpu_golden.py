"""GPU path (host C ABI) against the committed golden fixtures of the oracle.

Bars: LU pivots identical (ties included: the fixture with small-integer
entries has many exact ties, and the first maximum must win as in DDLA's
AMax); failing-pivot indices identical; factors, solutions and products
max-relative within 1e-12 of the oracle's (GEMM 1e-13)."""
import os

import numpy as np
import pytest

from helpers import rel_max

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "ddla_golden.npz"))


def sym(L):
    return L + np.tril(L, -1).T


def test_gemm_golden(ddla, g):
    Cm = g["gemm_c0"].copy()
    ddla.BlasProvider.GeMM(1.0, g["gemm_a"], g["gemm_b"], 0.5, Cm)
    assert rel_max(Cm, g["gemm_c"]) <= 1e-13
    Cm = g["gemmt_c0"].copy()
    ddla.BlasProvider.GeMMT(ddla.LOWER, -1.0, g["gemmt_a"], g["gemmt_b"], 1.0, Cm)
    assert rel_max(Cm, g["gemmt_c"]) <= 1e-13
    assert np.array_equal(np.triu(Cm, 1), np.triu(g["gemmt_c0"], 1))   # upper triangle untouched


def test_trsm_golden(ddla, g):
    X = g["trsm_b"].copy()
    ddla.BlasProvider.TrSM(ddla.LEFT, ddla.LOWER, ddla.NO_TRANSPOSE, ddla.UNIT, 1.0, g["trsm_a"], X)
    assert rel_max(X, g["trsm_x"]) <= 1e-12


@pytest.mark.parametrize("name", ["plu", "plutie"])
def test_plu_golden(ddla, g, name):
    F = g[f"{name}_a"].copy()
    piv = np.zeros(F.shape[0], dtype=np.int32)
    ddla.LU.PLUDecompose(F, piv)
    assert np.array_equal(piv, g[f"{name}_piv"])
    assert rel_max(F, g[f"{name}_f"]) <= 1e-12
    if name == "plu":
        x = g["plu_b"].copy()
        ddla.LU.PLUSolve(F, piv, x)
        assert rel_max(x, g["plu_x"]) <= 1e-12


def test_plu_singular_golden(ddla, g):
    with pytest.raises(ddla.LinalgError) as e:
        ddla.LU.PLUDecompose(g["plusing_a"].copy(), np.zeros(40, dtype=np.int32))
    assert e.value.index == int(g["plusing_info"])


def test_lu_nopiv_golden(ddla, g):
    F = g["lunp_a"].copy()
    ddla.LU.LUDecompose(F)
    assert rel_max(F, g["lunp_f"]) <= 1e-12


def test_cholesky_golden(ddla, g):
    A = sym(g["chol_a"])
    for name, uplo, tri in (("lo", ddla.LOWER, np.tril), ("up", ddla.UPPER, np.triu)):
        F = A.copy()
        ddla.Cholesky.CholDecompose(uplo, F)
        assert rel_max(tri(F), g[f"chol{name}_f"]) <= 1e-12
        X = g["chol_b"].copy()
        ddla.Cholesky.CholeskySolve(uplo, F, X)
        assert rel_max(X, g[f"chol{name}_x"]) <= 1e-12
    with pytest.raises(ddla.LinalgError) as e:
        ddla.Cholesky.CholDecompose(ddla.LOWER, g["cholfail_a"].copy())
    assert e.value.index == int(g["cholfail_info"])


def test_ldlt_golden(ddla, g):
    F = sym(g["ldlt_a"])
    ddla.LDLT.LDLTDecompose(ddla.LOWER, F)
    assert rel_max(np.tril(F), g["ldlt_f"]) <= 1e-12
    x = g["ldlt_b"].copy()
    ddla.LDLT.LDLTSolve(ddla.LOWER, F, x)
    assert rel_max(x, g["ldlt_x"]) <= 1e-12


@pytest.mark.parametrize("i,expr", [(1, "bik,bkj->bij"), (2, "abcd,cdef->abef"), (3, "iij,jk->ik")])
def test_einsum_golden(ddla, g, i, expr):
    from ddla_gb300 import einsum
    Cm = np.zeros_like(g[f"ein{i}_c"])
    einsum.Contract(Cm, expr, 1.0, g[f"ein{i}_l"], g[f"ein{i}_r"])
    assert rel_max(Cm, g[f"ein{i}_c"]) <= 1e-13


@pytest.fixture(scope="module")
def gn():
    return np.load(os.path.join(HERE, "golden", "ddla_golden_next.npz"))


def test_level3_next_golden(ddla, gn):
    nan_up = lambda x: x + np.triu(np.full(x.shape, np.nan), 1)      # noqa: E731
    Cm = gn["symm_c0"].copy()
    ddla.BlasProvider.SyMM(ddla.LEFT, ddla.LOWER, 1 / np.pi, nan_up(gn["symm_a"]), gn["symm_b"], np.e, Cm)
    assert rel_max(Cm, gn["symm_c"]) <= 1e-13
    A = gn["trmm_a"] + np.tril(np.full((45, 45), np.nan))
    X = gn["trmm_b"].copy()
    ddla.BlasProvider.TrMM(ddla.RIGHT, ddla.UPPER, ddla.TRANSPOSE, ddla.UNIT, 1.2, A, X)
    assert rel_max(X, gn["trmm_x"]) <= 1e-13
    Cm = gn["trmm3_c0"].copy()
    ddla.BlasProvider.TrMM3(ddla.LEFT, ddla.LOWER, ddla.NO_TRANSPOSE, ddla.NONUNIT, ddla.TRANSPOSE, 1.0,
                            nan_up(gn["trmm3_a"]), gn["trmm3_bt"], 1.0, Cm)
    assert rel_max(Cm, gn["trmm3_c"]) <= 1e-13
    Cm = gn["syr2k_c0"].copy()
    ddla.BlasProvider.SyR2k(ddla.UPPER, 1 / np.pi, gn["syr2k_a"], gn["syr2k_b"], np.e, Cm)
    assert rel_max(np.triu(Cm), gn["syr2k_c"]) <= 1e-13


@pytest.mark.parametrize("name", ["qr1", "qr2"])
def test_qr_golden(ddla, gn, name):
    A = gn[f"{name}_a"]
    m, n = A.shape
    F = A.copy()
    T = ddla.QR.QRDecompose(F)
    assert rel_max(np.triu(F), np.triu(gn[f"{name}_f"])) <= 1e-12
    assert rel_max(np.tril(F, -1), np.tril(gn[f"{name}_f"], -1)) <= 1e-11
    k = min(m, n)
    for j0 in range(0, k, T.shape[0]):
        b = min(T.shape[0], k - j0)
        assert rel_max(np.triu(T[:b, j0:j0 + b]), gn[f"{name}_t"][:b, j0:j0 + b]) <= 1e-11
    X = np.zeros((n, 2))
    ddla.QR.Solve(F, T, gn[f"{name}_b"], X)
    assert rel_max(X, gn[f"{name}_x"]) <= 1e-10
