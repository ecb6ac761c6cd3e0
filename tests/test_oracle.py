"""CPU pinning of the oracle (no GPU).

DDLA ships no golden vectors and cannot run here (C#/.NET, x86-only kernel,
closed Windows BLIS), so the oracle is pinned by (a) DDLA's own property tests
at their sizes and tolerances (Tests/TestFlame/*.cs,
Tests/TestEinsum/TestSimpleBSMTC.cs, Tests/TestManagedBlas/Level3m/*.cs) and
(b) an independent LAPACK/BLAS (scipy/numpy) on the same inputs, including the
exact partial-pivoting sequence.
"""
import numpy as np
import pytest
import scipy.linalg as sl

from helpers import apply_piv, berr, make_lmat, make_umat, norms, rel_max, rng, spd, uniform

TINY, SMALL, MEDIUM, LARGE = 4, 64, 256, 1024


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (7, 9, 5), (6, 8, 144), (130, 200, 300), (513, 600, 145)])
def test_gemm_matches_numpy(orc, m, n, k):
    # DDLA Tests/TestManagedBlas/Level3m/TestGeMM.cs:40-55: alpha=2, beta=1.2, abs tol 1e-10
    r = rng(10 + m)
    A, B, C0 = uniform(r, (m, k)), uniform(r, (k, n)), uniform(r, (m, n))
    Cm = C0.copy()
    orc.dgemm(2.0, A, B, 1.2, Cm)
    assert np.max(np.abs(Cm - (1.2 * C0 + 2.0 * A @ B))) < 1e-10


@pytest.mark.parametrize("layout", ["row", "col", "strided"])
def test_gemm_layouts(orc, layout):
    r = rng(3)
    m, n, k = 70, 90, 50
    def mk(shape):
        x = uniform(r, shape)
        if layout == "col":
            return np.asfortranarray(x)
        if layout == "strided":   # colStride = 4 (Tests/CreateUtils.cs)
            big = np.zeros((shape[0], shape[1] * 4))
            big[:, ::4] = x
            return big[:, ::4]
        return x
    A, B, Cm = mk((k, m)), mk((n, k)), mk((m, n))
    ref = 0.5 * Cm + 2.0 * A.T @ B.T
    orc.dgemm(2.0, A, B, 0.5, Cm, ta=orc.TRANS_T, tb=orc.TRANS_T)
    assert np.max(np.abs(Cm - ref)) < 1e-12


def test_gemm_beta_zero_ignores_nan(orc):
    A, B = np.ones((3, 2)), np.ones((2, 4))
    Cm = np.full((3, 4), np.nan)
    orc.dgemm(1.0, A, B, 0.0, Cm)
    assert np.all(Cm == 2.0)


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_gemmt_syrk(orc, uplo):
    # TestGeMMT.cs:94-112 / TestSyRk.cs:74-92
    r = rng(4)
    u = orc.LOWER if uplo == "L" else orc.UPPER
    tri = np.tril if uplo == "L" else np.triu
    anti = (lambda x: np.triu(x, 1)) if uplo == "L" else (lambda x: np.tril(x, -1))
    A, B, C0 = uniform(r, (300, 70)), uniform(r, (70, 300)), uniform(r, (300, 300))
    Cm = C0.copy()
    orc.dgemmt(u, 2.0, A, B, 1.2, Cm)
    assert np.max(np.abs(tri(Cm) - tri(1.2 * C0 + 2 * A @ B))) < 1e-10
    assert np.array_equal(anti(Cm), anti(C0))
    Cm = C0.copy()
    orc.dsyrk(u, -1.0, A, 1.0, Cm)
    assert np.max(np.abs(tri(Cm) - tri(C0 - A @ A.T))) < 1e-10


def _tri(X, uplo, diag):
    T = np.tril(X) if uplo == 0xC0 else np.triu(X)
    if diag:
        np.fill_diagonal(T, 1.0)
    return T


def _sym(X, uplo):
    L = np.tril(X) if uplo == 0xC0 else np.triu(X)
    return L + L.T - np.diag(np.diag(X))


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("uplo", [0xC0, 0x60])
@pytest.mark.parametrize("m,n", [(64, 64), (300, 64), (64, 300), (150, 151)])
def test_symm(orc, side, uplo, m, n):
    # TestSyMM.cs:40-69: alpha 1/pi, beta e, sizes small/large in both roles;
    # DDLA's bound is Nrm1(diff) <= 2e-5, this one is elementwise 1e-12.
    r = rng(20 + m + n)
    na = m if side == 0 else n
    A = uniform(r, (na, na))
    # the unreferenced triangle is garbage: it must never be read
    junk = np.triu(np.full((na, na), np.nan), 1) if uplo == 0xC0 else np.tril(np.full((na, na), np.nan), -1)
    As = np.where(np.isnan(junk), np.nan, A)
    B, C0 = uniform(r, (m, n)), uniform(r, (m, n))
    S = _sym(A, uplo)
    ref = np.e * C0 + (1 / np.pi) * (S @ B if side == 0 else B @ S)
    Cm = C0.copy()
    orc.dsymm(side, uplo, 1 / np.pi, As, B, np.e, Cm)
    assert np.max(np.abs(Cm - ref)) < 1e-12


@pytest.mark.parametrize("uplo", [0xC0, 0x60])
@pytest.mark.parametrize("ta,tb", [(0, 0), (8, 8), (0, 8)])
def test_syr2k(orc, uplo, ta, tb):
    # TestSyR2k.cs:24-40: m 512, k 260, alpha 1/pi, beta e
    r = rng(21)
    m, k = 512, 260
    A = uniform(r, (k, m) if ta else (m, k))
    B = uniform(r, (k, m) if tb else (m, k))
    opA, opB = (A.T if ta else A), (B.T if tb else B)
    C0 = uniform(r, (m, m))
    tri = np.tril if uplo == 0xC0 else np.triu
    anti = (lambda x: np.triu(x, 1)) if uplo == 0xC0 else (lambda x: np.tril(x, -1))
    Cm = C0.copy()
    orc.dsyr2k(uplo, 1 / np.pi, A, B, np.e, Cm, ta=ta, tb=tb)
    ref = np.e * C0 + (1 / np.pi) * (opA @ opB.T + opB @ opA.T)
    assert np.max(np.abs(tri(Cm) - tri(ref))) < 1e-11
    assert np.array_equal(anti(Cm), anti(C0))


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("uplo", [0xC0, 0x60])
@pytest.mark.parametrize("trans", [0, 8])
@pytest.mark.parametrize("diag", [0, 0x100])
def test_trmm_trmm3(orc, side, uplo, trans, diag):
    # TestTrMM.cs:195-207 (alpha 1.2, tol 1e-10) and TestTrMM3.cs:195-213
    # (alpha = beta = 1, tol 1e-10); square, rectangular here.
    r = rng(22)
    m, n = 200, 150
    na = m if side == 0 else n
    A = uniform(r, (na, na))
    opT = _tri(A, uplo, diag)
    opT = opT.T if trans else opT
    B = uniform(r, (m, n))
    X = B.copy()
    orc.dtrmm(side, uplo, trans, diag, 1.2, A, X)
    ref = 1.2 * (opT @ B if side == 0 else B @ opT)
    assert np.max(np.abs(X - ref)) < 1e-10
    C0 = uniform(r, (m, n))
    Cm = C0.copy()
    Bt = np.ascontiguousarray(B.T)
    orc.dtrmm3(side, uplo, trans, diag, 1.0, A, Bt, 1.0, Cm, tb=8)
    ref = C0 + (opT @ B if side == 0 else B @ opT)
    assert np.max(np.abs(Cm - ref)) < 1e-10


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("uplo", [0xC0, 0x60])
@pytest.mark.parametrize("trans", [0, 8])
@pytest.mark.parametrize("diag", [0, 0x100])
def test_trsm(orc, side, uplo, trans, diag):
    # TestTrSM.cs:105-127: diagonal shifted by 2, alpha 1.2, tol 1e-8
    r = rng(5)
    m, n = 300, 170
    na = m if side == 0 else n
    A = uniform(r, (na, na)) / na + 2 * np.eye(na)
    T = np.tril(A) if uplo == 0xC0 else np.triu(A)
    if diag:
        np.fill_diagonal(T, 1.0)
    opT = T.T if trans else T
    B = uniform(r, (m, n))
    X = B.copy()
    orc.dtrsm(side, uplo, trans, diag, 1.2, A, X)
    res = opT @ X - 1.2 * B if side == 0 else X @ opT - 1.2 * B
    assert np.max(np.abs(res)) < 1e-8


def test_damax_first_max_and_nan(orc):
    assert orc.damax(np.array([1.0, -3.0, 3.0, 2.0])) == 1
    assert orc.damax(np.array([np.nan, 0.5, -0.5])) == 1
    assert orc.damax(np.array([np.nan, np.nan])) == 0
    assert orc.damax(np.zeros(0)) == 0


@pytest.mark.parametrize("n", [TINY, SMALL, 127, 128, 129, MEDIUM])
def test_plu_property_and_lapack_pivots(orc, n):
    # TestPLU.cs:79-116: A = L*U from random unit-L/U, ||P*A - L*U|| < 1e-8, 20 repetitions
    r = rng(100 + n)
    for _ in range(5):
        A = make_lmat(r.random((n, n))) @ make_umat(r.random((n, n)))
        F = A.copy()
        info, piv = orc.dgetrf(F)
        assert info == 0
        L, U = make_lmat(F), make_umat(F)
        for v in norms(apply_piv(A, piv) - L @ U):
            assert v < 1e-8
    # independent LAPACK: identical partial-pivoting sequence on N(0,1) inputs
    # (the L*U inputs above are exponentially ill-conditioned, so their late
    # pivots are decided by rounding noise)
    for _ in range(5):
        A = r.standard_normal((n, n))
        F = A.copy()
        info, piv = orc.dgetrf(F)
        lu, sp = sl.lu_factor(A)
        assert np.array_equal(piv, sp - np.arange(n))
        assert rel_max(F, lu) < 1e-10


def test_plu_large_spd_and_solver(orc):
    # TestPLU.cs:22-73 (RandomSPD(1024), tol 1e-6; solver with X = I)
    r = rng(7)
    n = LARGE
    G = r.random((n, n))
    A = G @ G.T + n * np.eye(n)
    F = A.copy()
    info, piv = orc.dgetrf(F)
    assert info == 0
    for v in norms(apply_piv(A, piv) - make_lmat(F) @ make_umat(F)):
        assert v < 1e-6
    A = r.random((n, n))
    X = A.copy()
    info, piv = orc.dgetrf(X)
    B = A @ np.eye(n)
    orc.dgetrs(X, piv, B)
    for v in norms(B - np.eye(n)):
        assert v < 1e-6


@pytest.mark.parametrize("n", [TINY, SMALL, MEDIUM])
def test_lu_nopiv_property(orc, n):
    # TestLU.cs:31-63: tol 1e-6
    r = rng(200 + n)
    A = make_lmat(r.random((n, n))) @ make_umat(r.random((n, n)) + n * np.eye(n))
    F = A.copy()
    assert orc.dgetrf_nopiv(F) == 0
    for v in norms(A - make_lmat(F) @ make_umat(F)):
        assert v < 1e-6
    b = r.random((n, 3))
    x = b.copy()
    orc.dgetrs_nopiv(F, x)
    assert berr(A, x, b) < 1e-14
    x = b.copy()
    orc.dgetrs_nopiv(F, x, trans=1)
    assert berr(A.T, x, b) < 1e-14


@pytest.mark.parametrize("n", [TINY, SMALL, MEDIUM])
@pytest.mark.parametrize("uplo", ["L", "U"])
def test_cholesky_property(orc, n, uplo):
    # TestChol.cs:26-96: A = L*L^T (random L), tol 1e-10
    r = rng(300 + n)
    L0 = r.random((n, n))
    A = L0 @ L0.T if uplo == "L" else L0.T @ L0
    A += n * np.eye(n) * 1e-3
    F = A.copy()
    u = orc.LOWER if uplo == "L" else orc.UPPER
    assert orc.dpotrf(u, F) == 0
    if uplo == "L":
        Lf = np.tril(F)
        res = A - Lf @ Lf.T
    else:
        Uf = np.triu(F)
        res = A - Uf.T @ Uf
    for v in norms(res):
        assert v < 1e-10 * max(1.0, np.abs(A).max())
    ref = np.linalg.cholesky(A)
    got = np.tril(F) if uplo == "L" else np.triu(F).T
    assert rel_max(got, ref) < 1e-12


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_cholesky_solver(orc, uplo):
    # TestChol.cs:101-162: U*U^T + sqrt(n) I, 256 RHS, tol 1e-8
    r = rng(9)
    n = 300
    U = r.random((n, n))
    A = U @ U.T + np.sqrt(n) * np.eye(n)
    X = r.random((n, 64))
    B = A @ X
    F = A.copy()
    u = orc.LOWER if uplo == "L" else orc.UPPER
    assert orc.dpotrf(u, F) == 0
    orc.dpotrs(u, F, B)
    for v in norms(B - X):
        assert v < 1e-8


@pytest.mark.parametrize("n", [TINY, SMALL, MEDIUM])
@pytest.mark.parametrize("uplo", ["L", "U"])
def test_ldlt_property(orc, n, uplo):
    r = rng(400 + n)
    A = spd(r, n)
    F = A.copy()
    u = orc.LOWER if uplo == "L" else orc.UPPER
    assert orc.dldlt(u, F) == 0
    D = np.diag(np.diag(F))
    L = make_lmat(F) if uplo == "L" else make_lmat(F.T)
    for v in norms(A - L @ D @ L.T):
        assert v < 1e-10
    b = r.random((n, 4))
    x = b.copy()
    assert orc.dldlts(u, F, x) == 0
    assert berr(A, x, b) < 1e-14


def test_failures_report_pivot_index(orc):
    A = np.eye(5)
    A[2, 2] = -1.0
    assert orc.dpotrf(orc.LOWER, A.copy()) == 3
    S = np.eye(4)
    S[:, 1] = 0.0          # singular: column 1 is zero below the diagonal too
    info, _ = orc.dgetrf(S.copy())
    assert info == 2
    Z = np.eye(4)
    Z[1, 1] = 0.0
    assert orc.dldlt(orc.LOWER, Z.copy()) == 2


@pytest.mark.parametrize("expr,sa,sb", [
    ("mnk,nktc->mct", (5, 7, 9), (7, 9, 4, 3)),      # Tests/TestEinsum/TestSimpleBSMTC.cs:10-51
    ("mk,kn->mn", (37, 29), (29, 23)),
    ("bik,bkj->bij", (6, 20, 21), (6, 21, 22)),
    ("abcd,cdef->abef", (4, 5, 6, 7), (6, 7, 3, 2)),
    ("ij,jk->ki", (11, 13), (13, 17)),
    ("aij,ajk->ik", (3, 8, 9), (3, 9, 10)),           # batch mode summed (A-B shared, not in C)
])
def test_contract_vs_einsum(orc, expr, sa, sb):
    r = rng(11)
    A, B = uniform(r, sa), uniform(r, sb)
    ref = np.einsum(expr.replace(" ", ""), A, B)
    Cm = np.zeros(ref.shape)
    orc.contract(expr, 1.0, A, B, Cm)
    assert np.max(np.abs(Cm - ref)) < 1e-10


def test_contract_plan_folds_to_single_gemm(orc):
    A, B = np.zeros((8, 8, 8, 8)), np.zeros((8, 8, 8, 8))
    Cm = np.zeros((8, 8, 8, 8))
    d = orc.plan_dict(orc.contract_plan("abcd,cdef->abef", A, B, Cm))
    assert len(d["m"]) == 1 and len(d["n"]) == 1 and len(d["k"]) == 1 and d["batch"] == []
    assert d["m"][0][0] == 64 and d["n"][0][0] == 64 and d["k"][0][0] == 64


@pytest.mark.parametrize("m,n", [(TINY, TINY), (SMALL * 3 + 1, SMALL), (MEDIUM, MEDIUM), (MEDIUM * 3 + 1, MEDIUM),
                                 (600, 300), (200, 300)])
def test_qr_property_and_lapack(orc, m, n):
    # TestQR.cs:58-79: Q R = A with 1e-10 in the 1-, Frobenius and inf-norms
    r = rng(40 + m + n)
    A0 = uniform(r, (m, n))
    A = A0.copy()
    T = np.zeros((orc.qr_t_rows(m, n), n))
    orc.dgeqrf(A, T)
    Q = orc.dorgqr(A, T)
    R = np.triu(A)
    for nv in norms(Q @ R - A0):
        assert nv < 1e-10
    assert np.max(np.abs(Q.T @ Q - np.eye(m))) < 1e-13
    # LAPACK (scipy) uses the same sign rule (beta = -sign(alpha) |x|) and the
    # same vectors; it leaves a column with nothing below the diagonal alone
    # where DDLA reflects it (rho = -chi), so its last row of a square R differs
    # in sign.
    (raw, tau), _ = sl.qr(A0, mode="raw")
    k = min(m, n)
    kk = k - 1 if m <= n else k
    assert np.max(np.abs(np.triu(A)[:kk] - np.triu(raw)[:kk])) < 1e-12 * max(1.0, np.abs(raw).max())
    assert np.max(np.abs(np.tril(A, -1)[:, :kk] - np.tril(raw, -1)[:, :kk])) < 1e-11
    # T's diagonal blocks: tau_ddla = 1 / tau_lapack, S(i, j) = u_i^T u_j
    tb = T.shape[0]
    U = np.tril(A, -1)[:, :k] + np.eye(m, k)
    for j0 in range(0, k, tb):
        b = min(tb, k - j0)
        Ub = U[:, j0:j0 + b]
        S = Ub.T @ Ub
        np.fill_diagonal(S, np.diag(S) / 2)
        assert np.max(np.abs(np.triu(T[:b, j0:j0 + b]) - np.triu(S))) < 1e-12 * max(1.0, np.abs(S).max())


def test_qr_apply_and_solve(orc):
    # TestQR.cs:30-56: solve at 1e-6 (here 1024 x 1024 with 64 right-hand sides)
    r = rng(41)
    m, n, nrhs = 1024, 1024, 64
    A0 = uniform(r, (m, n))
    X0 = uniform(r, (n, nrhs))
    B = A0 @ X0
    A = A0.copy()
    T = np.zeros((orc.qr_t_rows(m, n), n))
    orc.dgeqrf(A, T)
    X = orc.dgeqrs(A, T, B)
    for nv in norms(X - X0):
        assert nv < 1e-6
    Y = B.copy()
    orc.dormqr(8, A, T, Y)                       # Q^T B
    Z = Y.copy()
    orc.dormqr(0, A, T, Z)                       # Q Q^T B = B
    assert np.max(np.abs(Z - B)) < 1e-10 * np.abs(B).max()
    assert np.max(np.abs(np.tril(Y[:n], -1) * 0 + Y[:n] - np.triu(A)[:n] @ X0)) < 1e-9 * np.abs(B).max()


def test_qr_least_squares_tall(orc):
    r = rng(42)
    m, n = 700, 300
    A0 = uniform(r, (m, n))
    B = uniform(r, (m, 3))
    A = A0.copy()
    T = np.zeros((orc.qr_t_rows(m, n), n))
    orc.dgeqrf(A, T)
    X = orc.dgeqrs(A, T, B)
    Xl = np.linalg.lstsq(A0, B, rcond=None)[0]
    assert np.max(np.abs(X - Xl)) < 1e-10


@pytest.mark.parametrize("n", [1, 2, 5, 64, 65, 150])
def test_tridiag_property_and_lapack(orc, n):
    # Tridiagonaling.Tridiag: Q^T A Q = tridiag(d, e) from the lower triangle;
    # the upper triangle is never read (NaN here).  LAPACK's dsytrd (uplo L)
    # makes the same reduction with reflectors of the opposite sign, so d
    # agrees and e agrees in magnitude.
    from scipy.linalg import lapack
    r = rng(80 + n)
    G = uniform(r, (n, n))
    S = G + G.T
    A = np.tril(S) + np.triu(np.full((n, n), np.nan), 1)
    T = np.zeros((orc.trd_t_rows(n), n))
    d, e = orc.dsytrd(A, T)
    Q = A
    Tr = np.diag(d) + np.diag(e, -1) + np.diag(e, 1)
    assert np.max(np.abs(Q.T @ S @ Q - Tr)) < 1e-12 * max(1.0, np.abs(S).max()) * max(n, 1) ** 0.5
    assert np.max(np.abs(Q.T @ Q - np.eye(n))) < 1e-13
    if n > 1:
        _, dl, el, _, info = lapack.dsytrd(S, lower=1)
        assert info == 0
        assert np.max(np.abs(d - dl)) < 1e-12 * max(1.0, np.abs(S).max()) * n ** 0.5
        assert np.max(np.abs(np.abs(e) - np.abs(el))) < 1e-12 * max(1.0, np.abs(S).max()) * n ** 0.5


@pytest.mark.parametrize("m,n", [(1, 1), (5, 5), (9, 4), (200, 130), (300, 300), (301, 260)])
def test_bidiag_property(orc, m, n):
    # Bidiagonaling.Bidiag2 (one stage): U^T A V = bidiag(d, e), U and V
    # orthogonal, singular values of the bidiagonal equal numpy's of A.
    # (scipy has no dgebrd, so this oracle is pinned by these properties.)
    r = rng(100 + m + n)
    A0 = uniform(r, (m, n))
    U, V, d, e, TU, TV = orc.bidiag(A0.copy())
    B = np.zeros((m, n))
    B[np.arange(n), np.arange(n)] = d
    if n > 1:
        B[np.arange(n - 1), np.arange(1, n)] = e
    assert np.max(np.abs(U.T @ A0 @ V - B)) < 1e-13 * max(m, 1)
    assert np.max(np.abs(U.T @ U - np.eye(m))) < 1e-13
    assert np.max(np.abs(V.T @ V - np.eye(n))) < 1e-13
    sv = np.sort(np.abs(np.linalg.svd(B, compute_uv=False)))
    assert np.max(np.abs(sv - np.sort(np.linalg.svd(A0, compute_uv=False)))) < 1e-12 * max(m, 1)


def test_batched_oracle_equals_item_calls(orc):
    """orc_batched (items in parallel) gives bit-identical factors, pivots and
    solutions to the per-item oracle calls, with threads on."""
    r = rng(77)
    sizes = [1, 2, 9, 64, 127, 128, 129, 200, 256, 31]
    kinds = [0, 1, 2, 0, 2, 0, 1, 2, 0, 1]
    mats, rhs = [], []
    for n, k in zip(sizes, kinds):
        mats.append(spd(r, n) if k == 2 else r.standard_normal((n, n)) + (n * np.eye(n) if k == 1 else 0))
        rhs.append(r.standard_normal(n))
    orc.set_threads(4)
    try:
        res, info = orc.batched(sizes, kinds, mats, rhs)
    finally:
        orc.set_threads(1)
    assert np.all(info == 0)
    for (F, x, piv), A, b, k in zip(res, mats, rhs, kinds):
        Fo, xo = A.copy(), b.copy().reshape(-1, 1)
        if k == 0:
            rc, po = orc.dgetrf(Fo)
            orc.dgetrs(Fo, po, xo)
            assert np.array_equal(piv, po)
        elif k == 1:
            orc.dgetrf_nopiv(Fo)
            orc.dgetrs_nopiv(Fo, xo)
        else:
            orc.dpotrf(0xC0, Fo)
            orc.dpotrs(0xC0, Fo, xo)
        assert np.array_equal(F, Fo) and np.array_equal(x, xo.ravel())


@pytest.mark.parametrize("m,n", [(5, 3), (7, 7), (33, 32), (64, 64), (95, 61), (131, 131), (300, 257)])
def test_bidiag2s_oracle_properties(orc, m, n):
    """The oracle's two-stage bidiagonal reduction (Bidiagonaling.Bidiag through
    TwoStageBidiag) pinned by properties, with the bars of DDLA's SVD tests
    (Tests/TestFlame/TestSVD.cs:31-72: reconstruction norms < 1e-10,
    orthogonality < 1e-8) and the singular values against LAPACK."""
    r = rng(m * 1000 + n)
    A = uniform(r, (m, n))
    W = A.copy()
    U, V, d, e = orc.bidiag2s(W)
    B = np.zeros((m, n))
    B[np.arange(n), np.arange(n)] = d
    if n > 1:
        B[np.arange(n - 1), np.arange(1, n)] = e
    for v in norms(A - U @ B @ V.T):
        assert v < 1e-10
    assert np.linalg.norm(U @ U.T - np.eye(m)) < 1e-8
    assert np.linalg.norm(V @ V.T - np.eye(n)) < 1e-8
    sv = np.sort(np.linalg.svd(B, compute_uv=False))
    ref = np.sort(np.linalg.svd(A, compute_uv=False))
    assert np.max(np.abs(sv - ref)) <= 1e-13 * ref.max()


def test_bidiag2s_oracle_band_after_stage_one(orc):
    """Same singular values as the one-stage reduction (Bidiag2) of the same
    matrix: both are orthogonal reductions of A."""
    r = rng(4242)
    A = uniform(r, (90, 70))
    U1, V1, d1, e1, _, _ = orc.bidiag(A.copy())
    U2, V2, d2, e2 = orc.bidiag2s(A.copy())

    def bd(d, e):
        B = np.diag(d)
        if len(e):
            B[np.arange(len(e)), np.arange(1, len(e) + 1)] = e
        return B
    s1 = np.sort(np.linalg.svd(bd(d1, e1), compute_uv=False))
    s2 = np.sort(np.linalg.svd(bd(d2, e2), compute_uv=False))
    assert np.max(np.abs(s1 - s2)) <= 1e-13 * s1.max()
