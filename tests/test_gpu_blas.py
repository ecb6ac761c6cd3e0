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


def _poison(A, uplo, unit=False, sym=False):
    """A copy of A whose unreferenced triangle (and, for a unit diagonal, the
    diagonal) is NaN: BLIS semantics say they are never read."""
    P = A.copy()
    mask = np.triu(np.ones(A.shape, bool), 1) if uplo == 0xC0 else np.tril(np.ones(A.shape, bool), -1)
    P[mask] = np.nan
    if unit:
        np.fill_diagonal(P, np.nan)
    return P


def _layout(x, layout):
    if layout == "col":
        return np.asfortranarray(x)
    if layout == "strided":
        big = np.zeros((x.shape[0], x.shape[1] * 3))
        big[:, ::3] = x
        return big[:, ::3]
    return x


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("uplo", [0xC0, 0x60])
@pytest.mark.parametrize("m,n", [(64, 64), (768, 64), (64, 768), (131, 9), (5, 300)])
def test_symm(ddla, orc, side, uplo, m, n):
    # DDLA TestSyMM.cs:40-69: alpha 1/pi, beta e; small and large in both roles
    r = rng(31 + m + 2 * n + side)
    na = m if side == 0 else n
    A = _poison(uniform(r, (na, na)), uplo)
    B, C0 = uniform(r, (m, n)), uniform(r, (m, n))
    Cg, Co = C0.copy(), C0.copy()
    ddla.BlasProvider.SyMM(side, uplo, 1 / np.pi, A, B, np.e, Cg)
    orc.dsymm(side, uplo, 1 / np.pi, A, B, np.e, Co)
    assert np.all(np.isfinite(Cg))
    assert rel_max(Cg, Co) <= 1e-13


@pytest.mark.parametrize("layout", ["row", "col", "strided"])
def test_symm_trans_b_layouts(ddla, orc, layout):
    r = rng(32)
    m, n = 150, 97
    A = _layout(_poison(uniform(r, (m, m)), 0x60), layout)
    Bt = _layout(uniform(r, (n, m)), layout)
    C0 = _layout(uniform(r, (m, n)), layout)
    Cg, Co = C0.copy(), C0.copy()
    ddla.BlasProvider.SyMM(0, 0x60, T, 0.7, A, Bt, 0.0, Cg)
    orc.dsymm(0, 0x60, 0.7, A, Bt, 0.0, Co, tb=T)
    assert rel_max(Cg, Co) <= 1e-13


@pytest.mark.parametrize("uplo", [0xC0, 0x60])
@pytest.mark.parametrize("ta,tb", [(N, N), (T, T), (N, T), (T, N)])
def test_syr2k(ddla, orc, uplo, ta, tb):
    # DDLA TestSyR2k.cs:24-40: m 512, k 260, alpha 1/pi, beta e
    r = rng(33 + ta + tb)
    m, k = 512, 260
    A = uniform(r, (k, m) if ta else (m, k))
    B = uniform(r, (k, m) if tb else (m, k))
    C0 = uniform(r, (m, m))
    Cg, Co = C0.copy(), C0.copy()
    ddla.BlasProvider.SyR2k(uplo, ta, tb, 1 / np.pi, A, B, np.e, Cg)
    orc.dsyr2k(uplo, 1 / np.pi, A, B, np.e, Co, ta=ta, tb=tb)
    assert rel_max(Cg, Co) <= 1e-13
    anti = (lambda x: np.triu(x, 1)) if uplo == 0xC0 else (lambda x: np.tril(x, -1))
    assert np.array_equal(anti(Cg), anti(C0))


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("uplo", [0xC0, 0x60])
@pytest.mark.parametrize("trans", [N, T])
@pytest.mark.parametrize("diag", [0, 0x100])
def test_trmm_all_variants(ddla, orc, side, uplo, trans, diag):
    # DDLA TestTrMM.cs:195-207: alpha 1.2, tol 1e-10 (here relative 1e-13)
    r = rng(34 + side + uplo + trans + diag)
    m, n = 300, 170
    na = m if side == 0 else n
    A = _poison(uniform(r, (na, na)), uplo, unit=bool(diag))
    B = uniform(r, (m, n))
    Xg, Xo = B.copy(), B.copy()
    ddla.BlasProvider.TrMM(side, uplo, trans, diag, 1.2, A, Xg)
    orc.dtrmm(side, uplo, trans, diag, 1.2, A, Xo)
    assert np.all(np.isfinite(Xg))
    assert rel_max(Xg, Xo) <= 1e-13


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("uplo", [0xC0, 0x60])
@pytest.mark.parametrize("trans", [N, T])
@pytest.mark.parametrize("diag", [0, 0x100])
@pytest.mark.parametrize("layout", ["row", "col"])
def test_trmm3_all_variants(ddla, orc, side, uplo, trans, diag, layout):
    # DDLA TestTrMM3.cs:195-213: alpha = beta = 1, tol 1e-10 (here relative 1e-13)
    r = rng(35 + side + uplo + trans + diag)
    m, n = 257, 130
    na = m if side == 0 else n
    A = _layout(_poison(uniform(r, (na, na)), uplo, unit=bool(diag)), layout)
    Bt = _layout(uniform(r, (n, m)), layout)
    C0 = _layout(uniform(r, (m, n)), layout)
    Cg, Co = C0.copy(), C0.copy()
    ddla.BlasProvider.TrMM3(side, uplo, trans, diag, T, 1.0, A, Bt, 1.0, Cg)
    orc.dtrmm3(side, uplo, trans, diag, 1.0, A, Bt, 1.0, Co, tb=T)
    assert rel_max(Cg, Co) <= 1e-13


def test_trmm_edges(ddla, orc):
    # empty, one element, thin (the 16-column tile) and alpha = 0
    ddla.BlasProvider.TrMM(0, 0xC0, 1.0, np.zeros((0, 0)), np.zeros((0, 5)))
    X = np.array([[3.0]])
    ddla.BlasProvider.TrMM(0, 0xC0, 2.0, np.array([[4.0]]), X)
    assert X[0, 0] == 24.0
    r = rng(36)
    A, B = uniform(r, (1000, 1000)), uniform(r, (1000, 7))
    Xg, Xo = B.copy(), B.copy()
    ddla.BlasProvider.TrMM(0, 0x60, T, 0x100, -0.5, A, Xg)
    orc.dtrmm(0, 0x60, T, 0x100, -0.5, A, Xo)
    assert rel_max(Xg, Xo) <= 1e-13
    Xg = B.copy()
    ddla.BlasProvider.TrMM(0, 0x60, 0.0, A, Xg)
    assert np.all(Xg == 0.0)


def test_structured_device_entry_points(ddla, orc):
    """The ddla_dev_* variants on device tensors (same kernels, no staging)."""
    torch = pytest.importorskip("torch")
    from ddla_gb300.device import Handle
    r = rng(37)
    m, n = 384, 200
    A = uniform(r, (m, m))
    B, C0 = uniform(r, (m, n)), uniform(r, (m, n))
    h = Handle(torch.cuda.current_stream())
    try:
        dA, dB, dC = (torch.tensor(x, device="cuda") for x in (A, B, C0))
        h.symm(0, 0xC0, 1.5, dA, dB, 0.25, dC)
        h.sync()
        Co = C0.copy()
        orc.dsymm(0, 0xC0, 1.5, A, B, 0.25, Co)
        assert rel_max(dC.cpu().numpy(), Co) <= 1e-13
        dX = dB.clone()
        h.trmm(0, 0x60, 0, 0, 2.0, dA, dX)
        h.sync()
        Xo = B.copy()
        orc.dtrmm(0, 0x60, 0, 0, 2.0, A, Xo)
        assert rel_max(dX.cpu().numpy(), Xo) <= 1e-13
        dC = torch.tensor(C0, device="cuda")
        h.trmm3(1, 0xC0, 8, 0x100, 1.0, dA[:n, :n], dB, -1.0, dC)
        h.sync()
        Co = C0.copy()
        orc.dtrmm3(1, 0xC0, 8, 0x100, 1.0, np.ascontiguousarray(A[:n, :n]), B, -1.0, Co)
        assert rel_max(dC.cpu().numpy(), Co) <= 1e-13
        dS = torch.tensor(uniform(r, (m, m)), device="cuda")
        S0 = dS.cpu().numpy()
        h.syr2k(0x60, 0.5, dA[:, :64], dB[:, :64], 2.0, dS)
        h.sync()
        So = S0.copy()
        orc.dsyr2k(0x60, 0.5, np.ascontiguousarray(A[:, :64]), np.ascontiguousarray(B[:, :64]), 2.0, So)
        assert rel_max(dS.cpu().numpy(), So) <= 1e-13
    finally:
        h.close()
