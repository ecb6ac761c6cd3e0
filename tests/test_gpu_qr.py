"""GPU parity of the Householder QR (ddla_dgeqrf / dormqr / dgeqrs / dorgqr)
against the oracle's restatement of DDLA's QR (DDLA/Factorizations/QR.cs),
through the C ABI.

Tolerances: R, the Householder vectors and the T factors element-wise within
1e-11 of the largest entry (FP64 on both sides, different reduction orders);
Q R = A within 1e-10 in the 1-, Frobenius and inf-norms (TestQR.cs:58-79);
solves within 1e-6 (TestQR.cs:30-56).
"""
import numpy as np
import pytest

from helpers import norms, rel_max, rng, uniform

pytestmark = pytest.mark.gpu


def _factor_both(ddla, orc, A0, t_rows=None):
    m, n = A0.shape
    tr = t_rows or orc.qr_t_rows(m, n)
    Ag, Tg = A0.copy(), np.zeros((tr, n))
    ddla.QR.QRDecompose(Ag, Tg)
    Ao, To = A0.copy(), np.zeros((tr, n))
    orc.dgeqrf(Ao, To)
    return Ag, Tg, Ao, To


def _check_factors(Ag, Tg, Ao, To):
    m, n = Ag.shape
    k = min(m, n)
    scale = max(1.0, np.abs(Ao).max())
    assert np.max(np.abs(np.triu(Ag) - np.triu(Ao))) <= 1e-11 * scale
    assert np.max(np.abs(np.tril(Ag, -1) - np.tril(Ao, -1))) <= 1e-11 * max(1.0, np.abs(np.tril(Ao, -1)).max())
    tb = Tg.shape[0]
    for j0 in range(0, k, tb):
        b = min(tb, k - j0)
        Sg, So = np.triu(Tg[:b, j0:j0 + b]), np.triu(To[:b, j0:j0 + b])
        assert np.max(np.abs(Sg - So)) <= 1e-11 * max(1.0, np.abs(So).max())


@pytest.mark.parametrize("m,n", [(4, 4), (193, 64), (256, 256), (769, 256), (600, 300), (200, 300), (1000, 513),
                                 (1, 1), (1, 7), (9, 1)])
def test_qr_matches_oracle(ddla, orc, m, n):
    r = rng(50 + m + 3 * n)
    A0 = uniform(r, (m, n))
    Ag, Tg, Ao, To = _factor_both(ddla, orc, A0)
    _check_factors(Ag, Tg, Ao, To)


@pytest.mark.parametrize("m,n", [(193, 64), (256, 256), (769, 256), (1024, 1024)])
def test_qr_deconstruct(ddla, m, n):
    # TestQR.cs:58-79: Q R = A, 1e-10 in three norms
    r = rng(51 + m)
    A0 = uniform(r, (m, n))
    Q, R = ddla.QR(A0).Deconstruct()
    for nv in norms(Q @ R - A0):
        assert nv < 1e-10
    assert np.max(np.abs(Q.T @ Q - np.eye(m))) < 1e-13


@pytest.mark.parametrize("t_rows", [64, 100, 256])
@pytest.mark.parametrize("layout", ["row", "col"])
def test_qr_t_layouts(ddla, orc, t_rows, layout):
    r = rng(52 + t_rows)
    A0 = uniform(r, (520, 330))
    if layout == "col":
        A0 = np.asfortranarray(A0)
    Ag, Tg, Ao, To = _factor_both(ddla, orc, A0, t_rows)
    _check_factors(Ag, Tg, Ao, To)
    Qg = np.zeros((520, 520))
    ddla.QR.FormQ(Ag, Tg, Qg)
    Qo = orc.dorgqr(Ao, To)
    assert rel_max(Qg, Qo) <= 1e-11


def test_qr_solve_large(ddla, orc):
    # TestQR.cs:30-56 (TestLargeBloQRSquareSolver): 1024 x 1024, tol 1e-6
    r = rng(53)
    m = n = 1024
    A0 = uniform(r, (m, n))
    X0 = uniform(r, (n, 64))
    B = A0 @ X0
    Xg = ddla.QR(A0).Solve(B)
    for nv in norms(Xg - X0):
        assert nv < 1e-6
    Ao, To = A0.copy(), np.zeros((256, n))
    orc.dgeqrf(Ao, To)
    Xo = orc.dgeqrs(Ao, To, B)
    assert rel_max(Xg, Xo) <= 1e-9


def test_qr_least_squares_and_apply(ddla, orc):
    r = rng(54)
    m, n = 3000, 700
    A0 = uniform(r, (m, n))
    B = uniform(r, (m, 5))
    qr = ddla.QR(A0)
    X = qr.Solve(B)
    Xl = np.linalg.lstsq(A0, B, rcond=None)[0]
    assert np.max(np.abs(X - Xl)) < 1e-10
    Y = B.copy()
    qr.ApplyQT(Y)
    Z = Y.copy()
    qr.ApplyQ(Z)
    assert np.max(np.abs(Z - B)) < 1e-12
    Ao, To = A0.copy(), np.zeros((256, n))
    orc.dgeqrf(Ao, To)
    Yo = B.copy()
    orc.dormqr(8, Ao, To, Yo)
    assert rel_max(Y, Yo) <= 1e-11


def test_qr_panel_paths(ddla, orc):
    """Narrow panels (qr.nb), and the in-place (through L2) panel kernel."""
    from ddla_gb300 import autotune as at
    r = rng(55)
    A0 = uniform(r, (900, 200))
    ref = None
    for table in ({}, {"qr.nb": 8}, {"qr.resident": 0}, {"qr.cluster": 2}):
        at.apply(table)
        try:
            Ag, Tg, Ao, To = _factor_both(ddla, orc, A0)
            _check_factors(Ag, Tg, Ao, To)
        finally:
            for k in table:
                at.tune_set(k, -(2 ** 63))
        if ref is None:
            ref = Ag
        assert rel_max(Ag, ref) <= 1e-12


def test_qr_tall_panel_and_device_entry(ddla):
    """A 50000 x 8 panel (too tall for shared memory at width 32) and the
    ddla_dev_* entry points on device tensors."""
    torch = pytest.importorskip("torch")
    from ddla_gb300.device import Handle
    r = rng(56)
    m, n = 50000, 8
    A0 = uniform(r, (m, n))
    h = Handle(torch.cuda.current_stream())
    try:
        dA = torch.tensor(A0, device="cuda")
        dT = torch.zeros(8, n, dtype=torch.float64, device="cuda")
        h.geqrf(dA, dT)
        dQ = torch.zeros(m, n, dtype=torch.float64, device="cuda")
        dQ[:n] = torch.eye(n, dtype=torch.float64, device="cuda")
        h.ormqr(False, dA, dT, dQ)         # thin Q = Q I(:, :n)
        h.sync()
        Q = dQ.cpu().numpy()
        R = np.triu(dA.cpu().numpy()[:n])
        assert np.max(np.abs(Q @ R - A0)) < 1e-12 * m ** 0.5
        B = uniform(r, (m, 2))
        dB = torch.tensor(B, device="cuda")
        dX = torch.zeros(n, 2, dtype=torch.float64, device="cuda")
        h.geqrs(dA, dT, dB, dX)
        h.sync()
        Xl = np.linalg.lstsq(A0, B, rcond=None)[0]
        assert np.max(np.abs(dX.cpu().numpy() - Xl)) < 1e-12
    finally:
        h.close()


def test_qr_argument_errors(ddla):
    with pytest.raises(ValueError):
        ddla.QR.QRDecompose(np.zeros((5, 4)), np.zeros((4, 3)))
    with pytest.raises(ValueError):
        ddla.QR.Solve(np.zeros((5, 4)), np.zeros((4, 4)), np.zeros((6, 1)), np.zeros((4, 1)))
    # m < n has no least-squares solve: the ABI rejects argument 2
    rc = ddla.lib().ddla_dgeqrs(3, 4, 1, None, 4, 1, None, 4, 4, 1, None, 1, 1, None, 1, 1)
    assert rc == -2


def test_qr_ozaki_block_reflectors(ddla, orc):
    """precision = DDLA_PREC_OZAKI: the large block-reflector products on the
    split-precision tensor-core GEMM; the factors stay within FP64-level
    distance of the oracle's and Q R = A."""
    r = rng(57)
    m, n = 1500, 1200
    A0 = uniform(r, (m, n))
    Ag, Tg = A0.copy(), np.zeros((256, n))
    ddla.QR.QRDecompose(Ag, Tg, precision=ddla.PREC_OZAKI)
    Ao, To = A0.copy(), np.zeros((256, n))
    orc.dgeqrf(Ao, To)
    assert np.max(np.abs(np.triu(Ag) - np.triu(Ao))) <= 1e-10 * np.abs(Ao).max()
    Q = np.zeros((m, m))
    ddla.QR.FormQ(Ag, Tg, Q)
    for nv in norms(Q @ np.triu(Ag) - A0):
        assert nv < 1e-9
