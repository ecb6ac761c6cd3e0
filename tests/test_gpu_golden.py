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
