"""GPU one-stage bidiagonal reduction (ddla_dbidiag) against the oracle's
restatement of DDLA's Bidiagonaling.Bidiag2 (DDLA/Transformations/
Bidiagonaling.cs:48-143).

Bars: d, e, U and V within 1e-11 (scaled) of the oracle's; U^T A V =
bidiag(d, e), U and V orthogonal, to FP64 accuracy."""
import numpy as np
import pytest

from helpers import rng, uniform

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n", [(1, 1), (2, 2), (5, 5), (9, 4), (200, 130), (300, 300), (301, 260), (700, 140)])
def test_bidiag_matches_oracle(ddla, orc, m, n):
    A0 = uniform(rng(110 + m + n), (m, n))
    Ug, Vg, dg, eg = ddla.Bidiagonaling.Bidiag2(A0.copy())
    Uo, Vo, do, eo, _, _ = orc.bidiag(A0.copy())
    tol = 1e-11 * max(m, 1)
    assert np.max(np.abs(dg - do)) <= tol
    if n > 1:
        assert np.max(np.abs(eg - eo)) <= tol
    assert np.max(np.abs(Ug - Uo)) <= tol
    assert np.max(np.abs(Vg - Vo)) <= tol
    B = np.zeros((m, n))
    B[np.arange(n), np.arange(n)] = dg
    if n > 1:
        B[np.arange(n - 1), np.arange(1, n)] = eg
    assert np.max(np.abs(Ug.T @ A0 @ Vg - B)) <= 1e-13 * max(m, 1)
    assert np.max(np.abs(Ug.T @ Ug - np.eye(m))) <= 1e-13
    assert np.max(np.abs(Vg.T @ Vg - np.eye(n))) <= 1e-13


def test_bidiag_col_major_and_errors(ddla, orc):
    A0 = np.asfortranarray(uniform(rng(111), (260, 180)))
    Ug, Vg, dg, eg = ddla.Bidiagonaling.Bidiag2(A0.copy(order="F"))
    Uo, Vo, do, eo, _, _ = orc.bidiag(np.ascontiguousarray(A0))
    assert np.max(np.abs(dg - do)) <= 1e-10 and np.max(np.abs(Vg - Vo)) <= 1e-10
    with pytest.raises(ValueError):
        ddla.Bidiagonaling.Bidiag2(np.zeros((3, 5)))


def test_bidiag_device_ozaki(ddla):
    torch = pytest.importorskip("torch")
    from ddla_gb300.device import Handle
    m, n = 1200, 900
    A0 = uniform(rng(112), (m, n))
    h = Handle(torch.cuda.current_stream())
    try:
        for prec in (0, ddla.PREC_OZAKI):
            dA = torch.tensor(A0, device="cuda")
            dd = torch.zeros(n, dtype=torch.float64, device="cuda")
            de = torch.zeros(n - 1, dtype=torch.float64, device="cuda")
            dU = torch.zeros(m, m, dtype=torch.float64, device="cuda")
            dV = torch.zeros(n, n, dtype=torch.float64, device="cuda")
            h.bidiag(dA, dd, de, dU, dV, precision=prec)
            h.sync()
            U, V, d, e = dU.cpu().numpy(), dV.cpu().numpy(), dd.cpu().numpy(), de.cpu().numpy()
            B = np.zeros((m, n))
            B[np.arange(n), np.arange(n)] = d
            B[np.arange(n - 1), np.arange(1, n)] = e
            assert np.max(np.abs(U.T @ A0 @ V - B)) <= 1e-11
            sv = np.sort(np.abs(np.linalg.svd(B[:n], compute_uv=False)))
            assert np.max(np.abs(sv - np.sort(np.linalg.svd(A0, compute_uv=False)))) <= 1e-11
    finally:
        h.close()
