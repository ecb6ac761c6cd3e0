"""GPU parity of the level-3 calls against the oracle (DDLA's managed GEMM
restated) through the C ABI, host-pointer entry points.

Tolerances: GEMM max|dC| / max|C| <= 1e-13 at K <= 2048 (FP64 on both sides,
different summation order); TRSM residual relative 1e-12.
"""
import numpy as np
import pytest

from helpers import rel_max, rng, uniform

pytestmark = pytest.mark.gpu

T, N = 8, 0


def _gemm_case(ddla, orc, m, n, k, ta, tb, alpha, beta, layout, seed):
    r = rng(seed)
    def mk(shape):
        x = uniform(r, shape)
        if layout == "col":
            return np.asfortranarray(x)
        if layout == "strided":
            big = np.zeros((shape[0], shape[1] * 4))
            big[:, ::4] = x
            return big[:, ::4]
        return x
    A = mk((k, m) if ta else (m, k))
    B = mk((n, k) if tb else (k, n))
    C0 = mk((m, n))
    Cg, Co = C0.copy(), C0.copy()
    ddla.BlasProvider.GeMM(ta, tb, alpha, A, B, beta, Cg)
    orc.dgemm(alpha, A, B, beta, Co, ta=ta, tb=tb)
    return Cg, Co


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (7, 9, 5), (64, 64, 64), (65, 63, 129), (300, 17, 200),
                                   (1024, 1024, 1024), (513, 2047, 700)])
def test_gemm_shapes(ddla, orc, m, n, k):
    Cg, Co = _gemm_case(ddla, orc, m, n, k, N, N, 1.0, 0.5, "row", m + n + k)
    assert rel_max(Cg, Co) <= 1e-13


@pytest.mark.parametrize("ta", [N, T])
@pytest.mark.parametrize("tb", [N, T])
@pytest.mark.parametrize("layout", ["row", "col", "strided"])
def test_gemm_trans_layouts(ddla, orc, ta, tb, layout):
    # DDLA TestGeMM.cs:12-55 (alpha=2, beta=1.2; row-major, col-major, strided)
    Cg, Co = _gemm_case(ddla, orc, 133, 71, 90, ta, tb, 2.0, 1.2, layout, 17)
    assert np.max(np.abs(Cg - Co)) < 1e-10
    assert rel_max(Cg, Co) <= 1e-13


def test_gemm_beta_zero_does_not_read_c(ddla):
    A, B = np.ones((5, 3)), np.ones((3, 7))
    Cm = np.full((5, 7), np.nan)
    ddla.BlasProvider.GeMM(1.0, A, B, 0.0, Cm)
    assert np.all(Cm == 3.0)


def test_gemm_empty_and_k0(ddla):
    Cm = np.ones((4, 4))
    ddla.BlasProvider.GeMM(1.0, np.zeros((4, 0)), np.zeros((0, 4)), 0.5, Cm)
    assert np.all(Cm == 1.0)      # DDLA returns early on k == 0 (DDLA/BLAS/3m.cs:21)
    ddla.BlasProvider.GeMM(1.0, np.zeros((0, 3)), np.zeros((3, 4)), 0.5, np.zeros((0, 4)))


def test_gemm_shape_mismatch_raises(ddla):
    with pytest.raises(ValueError):
        ddla.BlasProvider.GeMM(1.0, np.zeros((3, 4)), np.zeros((5, 2)), 0.0, np.zeros((3, 2)))


@pytest.mark.parametrize("uplo", [0xC0, 0x60])
@pytest.mark.parametrize("m,k", [(300, 70), (129, 128), (1000, 64)])
def test_gemmt_and_syrk(ddla, orc, uplo, m, k):
    r = rng(m + k)
    A, B, C0 = uniform(r, (m, k)), uniform(r, (k, m)), uniform(r, (m, m))
    Cg, Co = C0.copy(), C0.copy()
    ddla.BlasProvider.GeMMT(uplo, 2.0, A, B, 1.2, Cg)
    orc.dgemmt(uplo, 2.0, A, B, 1.2, Co)
    assert rel_max(Cg, Co) <= 1e-13
    anti = (lambda x: np.triu(x, 1)) if uplo == 0xC0 else (lambda x: np.tril(x, -1))
    assert np.array_equal(anti(Cg), anti(C0))          # the other triangle is untouched
    Cg, Co = C0.copy(), C0.copy()
    ddla.BlasProvider.SyRk(uplo, -1.0, A, 1.0, Cg)
    orc.dsyrk(uplo, -1.0, A, 1.0, Co)
    assert rel_max(Cg, Co) <= 1e-13
    assert np.array_equal(anti(Cg), anti(C0))


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("uplo", [0xC0, 0x60])
@pytest.mark.parametrize("trans", [N, T])
@pytest.mark.parametrize("diag", [0, 0x100])
def test_trsm_all_variants(ddla, orc, side, uplo, trans, diag):
    # DDLA TestTrSM.cs:105-127: diag shifted by 2, alpha 1.2, tol 1e-8
    r = rng(side * 7 + uplo + trans + diag)
    m, n = 300, 170
    na = m if side == 0 else n
    A = uniform(r, (na, na)) / na + 2 * np.eye(na)
    B = uniform(r, (m, n))
    Xg, Xo = B.copy(), B.copy()
    ddla.BlasProvider.TrSM(side, uplo, trans, diag, 1.2, A, Xg)
    orc.dtrsm(side, uplo, trans, diag, 1.2, A, Xo)
    assert rel_max(Xg, Xo) <= 1e-12
    Tm = np.tril(A) if uplo == 0xC0 else np.triu(A)
    if diag:
        np.fill_diagonal(Tm, 1.0)
    opT = Tm.T if trans else Tm
    res = opT @ Xg - 1.2 * B if side == 0 else Xg @ opT - 1.2 * B
    assert np.max(np.abs(res)) < 1e-8
