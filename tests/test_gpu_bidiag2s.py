"""GPU two-stage bidiagonal reduction (ddla_dbidiag_twostage) against the
oracle's restatement of DDLA's Bidiagonaling.Bidiag through TwoStageBidiag
(DDLA/Transformations/Bidiagonaling.cs:14-33, 334-582).

Both run the same steps (blocked QR / LQ to a band of width 32, then the
band chase); the GPU runs the chase's cycles concurrently and stage 1 with
its own reduction orders, so agreement is to rounding: d, e, U and V within
1e-10 (scaled) of the oracle's.  U^T A V = bidiag(d, e) and the
orthogonality of U and V with DDLA's SVD-test bars
(Tests/TestFlame/TestSVD.cs:31-72) tightened to FP64 accuracy."""
import numpy as np
import pytest

from helpers import rng, uniform

pytestmark = pytest.mark.gpu


def _bd(m, n, d, e):
    B = np.zeros((m, n))
    B[np.arange(n), np.arange(n)] = d
    if n > 1:
        B[np.arange(n - 1), np.arange(1, n)] = e
    return B


@pytest.mark.parametrize("m,n", [(1, 1), (2, 2), (5, 3), (7, 7), (33, 32), (34, 33), (64, 64), (95, 61), (131, 131),
                                 (300, 257), (400, 96), (513, 513)])
def test_bidiag2s_matches_oracle(ddla, orc, m, n):
    A0 = uniform(rng(m * 1000 + n), (m, n))
    Ug, Vg, dg, eg = ddla.Bidiagonaling.Bidiag(A0)
    Uo, Vo, do, eo = orc.bidiag2s(A0.copy())
    tol = 1e-10 * max(m, 1)
    assert np.max(np.abs(dg - do)) <= tol
    if n > 1:
        assert np.max(np.abs(eg - eo)) <= tol
    assert np.max(np.abs(Ug - Uo)) <= tol
    assert np.max(np.abs(Vg - Vo)) <= tol
    assert np.max(np.abs(Ug.T @ A0 @ Vg - _bd(m, n, dg, eg))) <= 1e-13 * max(m, 1)
    assert np.max(np.abs(Ug.T @ Ug - np.eye(m))) <= 1e-13
    assert np.max(np.abs(Vg.T @ Vg - np.eye(n))) <= 1e-13


def test_bidiag2s_leaves_input_and_layouts(ddla, orc):
    # DDLA's Bidiag works on a clone: the input is not written; a column-major
    # input gives the row-major input's results
    A0 = uniform(rng(9001), (260, 180))
    A = A0.copy()
    Ug, Vg, dg, eg = ddla.Bidiagonaling.Bidiag(A)
    assert np.array_equal(A, A0)
    Uf, Vf, df, ef = ddla.Bidiagonaling.Bidiag(np.asfortranarray(A0))
    assert np.max(np.abs(df - dg)) <= 1e-11 and np.max(np.abs(Vf - Vg)) <= 1e-11
    with pytest.raises(ValueError):
        ddla.Bidiagonaling.Bidiag(np.zeros((3, 5)))


def test_bidiag2s_device_sizes_and_ozaki(ddla, orc):
    """Device entry point at a larger size: properties for FP64 and for the
    split-precision block-reflector products; the oracle's d and e (FP64),
    LAPACK's singular values (split precision)."""
    torch = pytest.importorskip("torch")
    from ddla_gb300.device import Handle
    m, n = 1500, 1100
    A0 = uniform(rng(9002), (m, n))
    _, _, do, eo = orc.bidiag2s(A0.copy())
    h = Handle(torch.cuda.current_stream())
    try:
        for prec in (0, ddla.PREC_OZAKI):
            dA = torch.tensor(A0, device="cuda")
            dd = torch.zeros(n, dtype=torch.float64, device="cuda")
            de = torch.zeros(n - 1, dtype=torch.float64, device="cuda")
            dU = torch.zeros(m, m, dtype=torch.float64, device="cuda")
            dV = torch.zeros(n, n, dtype=torch.float64, device="cuda")
            h.bidiag_twostage(dA, dd, de, dU, dV, precision=prec)
            h.sync()
            U, V, d, e = dU.cpu().numpy(), dV.cpu().numpy(), dd.cpu().numpy(), de.cpu().numpy()
            # split-precision products carry errors near 1e-14 relative per product
            bar = 1e-13 if prec == 0 else 1e-11
            assert np.max(np.abs(U.T @ A0 @ V - _bd(m, n, d, e))) <= bar * (m if prec == 0 else 1)
            assert np.max(np.abs(U.T @ U - np.eye(m))) <= bar
            assert np.max(np.abs(V.T @ V - np.eye(n))) <= bar
            if prec == 0:
                assert np.max(np.abs(d - do)) <= 1e-9 and np.max(np.abs(e - eo)) <= 1e-9
            else:
                # the bidiagonal entries move with the products' rounding through
                # the chase; the singular values do not
                sv = np.sort(np.linalg.svd(_bd(n, n, d, e), compute_uv=False))
                assert np.max(np.abs(sv - np.sort(np.linalg.svd(A0, compute_uv=False)))) <= 1e-11 * sv.max()
    finally:
        h.close()
