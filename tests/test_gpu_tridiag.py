"""GPU tridiagonal reduction (ddla_dsytrd) against the oracle's restatement
of DDLA's Tridiagonaling.Tridiag (DDLA/Transformations/Tridiagonaling.cs).

Bars: d, e, Q and the T factors within 1e-11 of the oracle's (relative to
the largest entry; FP64 on both sides, different reduction orders);
Q^T A Q = tridiag(d, e) and Q^T Q = I to FP64 accuracy.  The upper triangle
of A is NaN: it must never be read."""
import numpy as np
import pytest

from helpers import rel_max, rng, uniform

pytestmark = pytest.mark.gpu


def _sym(n, seed):
    G = uniform(rng(seed), (n, n))
    return G + G.T


@pytest.mark.parametrize("n", [1, 2, 3, 64, 65, 130, 300])
def test_tridiag_matches_oracle(ddla, orc, n):
    S = _sym(n, 90 + n)
    A = np.tril(S) + np.triu(np.full((n, n), np.nan), 1)
    Ag, Ao = A.copy(), A.copy()
    Tg, dg, eg = ddla.Tridiagonaling.Tridiag(Ag)
    To = np.zeros((orc.trd_t_rows(n), n))
    do, eo = orc.dsytrd(Ao, To)
    scale = max(1.0, np.abs(S).max())
    assert np.max(np.abs(dg - do)) <= 1e-11 * scale * n
    if n > 1:
        assert np.max(np.abs(eg - eo)) <= 1e-11 * scale * n
    assert np.max(np.abs(Ag - Ao)) <= 1e-11 * n
    tb = Tg.shape[0]
    for j0 in range(0, n - 1, tb):
        b = min(tb, n - 1 - j0)
        Sg, So = np.triu(Tg[:b, j0:j0 + b]), np.triu(To[:b, j0:j0 + b])
        assert np.max(np.abs(Sg - So)) <= 1e-10 * max(1.0, np.abs(So).max())
    Tr = np.diag(dg) + np.diag(eg, -1) + np.diag(eg, 1)
    assert np.max(np.abs(Ag.T @ S @ Ag - Tr)) <= 1e-12 * scale * n
    assert np.max(np.abs(Ag.T @ Ag - np.eye(n))) <= 1e-13 * max(n, 1) ** 0.5


@pytest.mark.parametrize("layout", ["col", "strided"])
def test_tridiag_layouts(ddla, orc, layout):
    n = 200
    S = _sym(n, 91)
    A = np.tril(S) + np.triu(np.full((n, n), np.nan), 1)
    if layout == "col":
        Ag = np.asfortranarray(A)
    else:
        big = np.full((n, 2 * n), 7.0)
        big[:, ::2] = A
        Ag = big[:, ::2]
    _, dg, eg = ddla.Tridiagonaling.Tridiag(Ag)
    do, eo = orc.dsytrd(A.copy(), np.zeros((64, n)))
    assert rel_max(dg, do) <= 1e-11 and rel_max(eg, eo) <= 1e-11
    if layout == "strided":
        assert np.all(big[:, 1::2] == 7.0)


def test_tridiag_device_large_and_ozaki(ddla):
    torch = pytest.importorskip("torch")
    from ddla_gb300.device import Handle
    n = 1500
    S = _sym(n, 92)
    h = Handle(torch.cuda.current_stream())
    try:
        for prec in (0, ddla.PREC_OZAKI):
            dA = torch.tensor(np.tril(S), device="cuda")
            dT = torch.zeros(64, n, dtype=torch.float64, device="cuda")
            dd = torch.zeros(n, dtype=torch.float64, device="cuda")
            de = torch.zeros(n - 1, dtype=torch.float64, device="cuda")
            h.sytrd(dA, dT, dd, de, precision=prec)
            h.sync()
            Q, d, e = dA.cpu().numpy(), dd.cpu().numpy(), de.cpu().numpy()
            Tr = np.diag(d) + np.diag(e, -1) + np.diag(e, 1)
            assert np.max(np.abs(Q.T @ S @ Q - Tr)) <= 1e-11 * np.abs(S).max() * n ** 0.5
            assert np.max(np.abs(Q.T @ Q - np.eye(n))) <= 1e-12
            ev = np.linalg.eigvalsh(S)
            assert np.max(np.abs(np.linalg.eigvalsh(Tr) - ev)) <= 1e-12 * np.abs(ev).max() * n ** 0.5
    finally:
        h.close()
