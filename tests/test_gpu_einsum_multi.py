"""GPU multi-operand einsum (ddla_einsum / ddla_dev_einsum) against the
oracle's pairwise restatement (same path, DDLA's MArray.Contract per step)
and numpy.einsum.  Bar: max-relative 1e-13 (FP64 DMMA products, different
summation order); Ozaki within 1e-14 relative to |A||B|-scaled magnitudes."""
import numpy as np
import pytest

from helpers import rel_max, rng, uniform
from test_einsum_multi import CASES

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("expr,shapes", CASES)
def test_einsum_matches_oracle(ddla, orc, expr, shapes):
    from ddla_gb300 import einsum as es
    r = rng(70 + len(expr))
    ops = [uniform(r, s) for s in shapes]
    got = es.Einsum(expr, *ops)
    ref = orc.einsum(expr, ops)
    assert rel_max(np.asarray(got), np.asarray(ref)) <= 1e-13
    assert np.max(np.abs(got - np.einsum(expr, *ops))) <= 1e-12 * max(1.0, np.abs(ref).max())


def test_einsum_alpha_beta_strided(ddla):
    from ddla_gb300 import einsum as es
    r = rng(71)
    A = uniform(r, (30, 40))[:, ::2]          # strided view, 30 x 20
    B = np.asfortranarray(uniform(r, (20, 25)))
    Cm = uniform(r, (25, 7))
    out0 = uniform(r, (30, 7))
    out = out0.copy()
    es.Einsum("ij,jk,kl->il", A, B, Cm, alpha=0.5, out=out, beta=1.0)   # DDLA's Einsum(result, expr, alpha, ...)
    ref = out0 + 0.5 * A @ B @ Cm
    assert np.max(np.abs(out - ref)) <= 1e-12
    big = np.zeros((30, 14))
    view = big[:, ::2]
    es.Einsum("ij,jk,kl->il", A, B, Cm, out=view, beta=0.0)
    assert np.max(np.abs(view - A @ B @ Cm)) <= 1e-12
    assert np.all(big[:, 1::2] == 0.0)


@pytest.mark.parametrize("expr,shape", [("ij->ji", (5, 7)), ("ii->i", (6, 6)), ("ijk->", (3, 4, 5)),
                                        ("ij->ij", (4, 4))])
def test_einsum_single_operand(ddla, expr, shape):
    from ddla_gb300 import einsum as es
    x = uniform(rng(72), shape)
    assert np.max(np.abs(es.Einsum(expr, x) - np.einsum(expr, x))) <= 1e-13


def test_dev_einsum_chain_and_ozaki(ddla, orc):
    torch = pytest.importorskip("torch")
    from ddla_gb300 import einsum as es
    from ddla_gb300.device import Handle
    r = rng(73)
    expr, shapes = "ab,bc,cd,de->ae", [(64, 300), (300, 256), (256, 200), (200, 48)]
    ops = [uniform(r, s) for s in shapes]
    ref = orc.einsum(expr, ops)
    h = Handle(torch.cuda.current_stream())
    try:
        dops = [torch.tensor(x, device="cuda") for x in ops]
        out = torch.zeros(64, 48, dtype=torch.float64, device="cuda")
        es.dev_einsum(h, expr, dops, out)
        h.sync()
        assert rel_max(out.cpu().numpy(), ref) <= 1e-13
        out.zero_()
        es.dev_einsum(h, expr, dops, out, precision=ddla.PREC_OZAKI)
        h.sync()
        assert rel_max(out.cpu().numpy(), ref) <= 1e-12
    finally:
        h.close()
