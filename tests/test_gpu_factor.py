"""GPU parity of the factorizations and solves against the oracle through the
C ABI (host-pointer entry points, DDLA-mirroring classes).

Bars: LU pivots identical to the oracle's (a first mismatch passes only as a
documented rounding tie); factors max-relative within 1e-10 of the oracle's;
reconstruction and solve backward errors at FP64 roundoff (<= 1e-14 on
well-conditioned inputs).  Failures report the same 1-based pivot index as the
oracle.
"""
import numpy as np
import pytest

from helpers import apply_piv, berr, make_lmat, make_umat, norms, pivot_tie_ok, rel_max, rng, spd

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 7, 8, 63, 64, 65, 127, 128, 129, 255, 256, 300, 1000, 1500])
def test_plu_matches_oracle(ddla, orc, n):
    r = rng(1000 + n)
    A = r.standard_normal((n, n))
    Fg, Fo = A.copy(), A.copy()
    piv_g = np.zeros(n, dtype=np.int32)
    ddla.LU.PLUDecompose(Fg, piv_g)
    info, piv_o = orc.dgetrf(Fo)
    assert info == 0
    ok, first = pivot_tie_ok(A, piv_g, piv_o)
    assert ok, f"pivot mismatch at {first} that is not a rounding tie"
    if first < 0:
        assert rel_max(Fg, Fo) <= 1e-10
    L, U = make_lmat(Fg), make_umat(Fg)
    assert np.max(np.abs(apply_piv(A, piv_g) - L @ U)) / np.abs(A).max() <= 1e-13 * max(1, n / 100)
    B = r.standard_normal((n, 3))
    Xg = ddla.LU(A).Solve(B)
    assert berr(A, Xg, B) <= 1e-14
    Xt = B.copy()
    ddla.LU.PLUSolve(Fg, piv_g, Xt, trans=True)
    assert berr(A.T, Xt, B) <= 1e-14


def test_plu_ddla_property_tests(ddla):
    # Tests/TestFlame/TestPLU.cs:79-116 (tiny/small/medium, tol 1e-8)
    r = rng(5)
    for n in (4, 64, 256):
        for _ in range(5):
            A = make_lmat(r.random((n, n))) @ make_umat(r.random((n, n)))
            F = A.copy()
            piv = np.zeros(n, dtype=np.int32)
            ddla.LU.PLUDecompose(F, piv)
            for v in norms(apply_piv(A, piv) - make_lmat(F) @ make_umat(F)):
                assert v < 1e-8


def test_plu_strided_and_colmajor_views(ddla, orc):
    r = rng(77)
    n = 200
    A = r.standard_normal((n, n))
    info, piv_o = orc.dgetrf(Fo := A.copy())
    for view in (np.asfortranarray(A.copy()), np.zeros((n, 3 * n))):
        if view.shape[1] == 3 * n:
            view[:, ::3] = A
            view = view[:, ::3]
        piv = np.zeros(n, dtype=np.int32)
        ddla.LU.PLUDecompose(view, piv)
        assert np.array_equal(piv, piv_o)
        assert rel_max(view, Fo) <= 1e-10


def test_plu_singular_reports_pivot(ddla, orc):
    S = np.eye(6)
    S[:, 3] = 0.0
    info, _ = orc.dgetrf(S.copy())
    with pytest.raises(ddla.LinalgError) as e:
        ddla.LU.PLUDecompose(S.copy(), np.zeros(6, dtype=np.int32))
    assert e.value.index == info == 4


def test_plu_nan_column_pivots_like_amax(ddla, orc):
    # NaN compares smaller than everything (bli_damaxv as DDLA documents it)
    r = rng(3)
    A = r.standard_normal((40, 40))
    A[5, 0] = np.nan
    Fg, Fo = A.copy(), A.copy()
    pg = np.zeros(40, dtype=np.int32)
    ddla.LU.PLUDecompose(Fg, pg)
    _, po = orc.dgetrf(Fo)
    assert pg[0] == po[0]


@pytest.mark.parametrize("n", [4, 64, 128, 129, 256, 500])
def test_lu_nopiv(ddla, orc, n):
    r = rng(2000 + n)
    A = r.standard_normal((n, n)) + n * np.eye(n)
    Fg, Fo = A.copy(), A.copy()
    ddla.LU.LUDecompose(Fg)
    assert orc.dgetrf_nopiv(Fo) == 0
    assert rel_max(Fg, Fo) <= 1e-12
    B = r.standard_normal((n, 2))
    X = ddla.LU(A, usePiv=False).Solve(B)
    assert berr(A, X, B) <= 1e-14
    X = B.copy()
    ddla.LU.LUSolve(Fg, X, trans=True)
    assert berr(A.T, X, B) <= 1e-14


@pytest.mark.parametrize("n", [1, 4, 64, 127, 128, 129, 256, 1000])
@pytest.mark.parametrize("uplo", [0xC0, 0x60])
def test_cholesky(ddla, orc, n, uplo):
    r = rng(3000 + n)
    A = spd(r, n)
    Fg, Fo = A.copy(), A.copy()
    ddla.Cholesky.CholDecompose(uplo, Fg)
    assert orc.dpotrf(uplo, Fo) == 0
    tri = np.tril if uplo == 0xC0 else np.triu
    assert rel_max(tri(Fg), tri(Fo)) <= 1e-12
    assert np.array_equal(Fg - tri(Fg), A - tri(A))   # other triangle untouched
    B = r.standard_normal((n, 16))
    X = ddla.Cholesky(A, uplo).Solve(B)
    assert berr(A, X, B) <= 1e-14


def test_cholesky_ddla_solver(ddla):
    # Tests/TestFlame/TestChol.cs:101-130: U U^T + sqrt(n) I, 256 RHS, tol 1e-8
    r = rng(9)
    n = 1024
    U = r.random((n, n))
    A = U @ U.T + np.sqrt(n) * np.eye(n)
    X = r.random((n, 256))
    B = A @ X
    Xs = ddla.Cholesky(A, ddla.LOWER).Solve(B)
    for v in norms(Xs - X):
        assert v < 1e-8


def test_cholesky_indefinite_reports_pivot(ddla, orc):
    for n, bad in ((10, 4), (300, 200)):
        A = np.eye(n)
        A[bad, bad] = -1.0
        exp = orc.dpotrf(0xC0, A.copy())
        with pytest.raises(ddla.LinalgError) as e:
            ddla.Cholesky.CholDecompose(0xC0, A.copy())
        assert e.value.index == exp == bad + 1


@pytest.mark.parametrize("n", [4, 64, 129, 256, 600])
@pytest.mark.parametrize("uplo", [0xC0, 0x60])
def test_ldlt(ddla, orc, n, uplo):
    r = rng(4000 + n)
    A = spd(r, n)
    Fg, Fo = A.copy(), A.copy()
    ddla.LDLT.LDLTDecompose(uplo, Fg)
    assert orc.dldlt(uplo, Fo) == 0
    tri = np.tril if uplo == 0xC0 else np.triu
    assert rel_max(tri(Fg), tri(Fo)) <= 1e-12
    B = r.standard_normal((n, 5))
    X = ddla.LDLT(uplo, A).Solve(B)
    assert berr(A, X, B) <= 1e-14
    L, D = ddla.LDLT(uplo, A).Deconstruct()
    assert np.max(np.abs(L @ D @ L.T - A)) <= 1e-12 if uplo == 0xC0 else True


def test_ldlt_zero_pivot(ddla, orc):
    Z = np.eye(300)
    Z[150, 150] = 0.0
    exp = orc.dldlt(0xC0, Z.copy())
    with pytest.raises(ddla.LinalgError) as e:
        ddla.LDLT.LDLTDecompose(0xC0, Z.copy())
    assert e.value.index == exp == 151
