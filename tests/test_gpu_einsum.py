"""GPU parity of MArray.Contract against the oracle's block-scatter
contraction and numpy (Tests/TestEinsum/TestSimpleBSMTC.cs, abs tol 1e-10)."""
import numpy as np
import pytest

from helpers import rng, uniform

pytestmark = pytest.mark.gpu

CASES = [
    ("mnk,nktc->mct", (15, 17, 19), (17, 19, 14, 13)),      # TestTC, dims in [14, 37)
    ("mk,kn->mn", (1025, 257), (257, 257)),                  # TestMM
    ("mk,kn->mn", (512, 144), (144, 513)),                   # TestMMFast: (mc+2) x (nc+1) x kc
    ("bik,bkj->bij", (8, 64, 48), (8, 48, 40)),              # batched
    ("abcd,cdef->abef", (8, 8, 8, 8), (8, 8, 8, 8)),          # folds to one GEMM
    ("ij,jk->ki", (40, 33), (33, 21)),                        # transposed output
    ("aij,ajk->ik", (3, 30, 20), (3, 20, 10)),                # shared mode summed
    ("abc,cb->a", (7, 6, 5), (5, 6)),                         # multi-mode K, gather path
    ("ii,ij->j", (9, 9), (9, 4)),                             # repeated symbol (diagonal)
    ("ab,c->abc", (6, 5), (4,)),                              # outer product
    ("acb,bd->adc", (5, 6, 7), (7, 8)),                       # permuted, non-foldable
]


@pytest.mark.parametrize("expr,sa,sb", CASES)
def test_contract_matches_oracle(ddla, orc, expr, sa, sb):
    from ddla_gb300 import einsum
    r = rng(hash(expr) % 1000)
    A, B = uniform(r, sa), uniform(r, sb)
    ref = np.einsum(expr, A, B)
    got = einsum.Contract(expr, 1.0, A, B)
    Co = np.zeros(ref.shape)
    orc.contract(expr, 1.0, A, B, Co)
    assert np.max(np.abs(got - ref)) < 1e-10
    assert np.max(np.abs(got - Co)) / max(np.abs(Co).max(), 1e-300) < 1e-13


def test_contract_accumulates_and_scales(ddla):
    from ddla_gb300 import einsum
    r = rng(5)
    A, B = uniform(r, (20, 30)), uniform(r, (30, 10))
    C0 = uniform(r, (20, 10))
    Cm = C0.copy()
    einsum.Contract(Cm, "mk,kn->mn", 2.0, A, B)
    assert np.max(np.abs(Cm - (C0 + 2.0 * A @ B))) < 1e-12
    Cm = C0.copy()
    einsum.Contract(0.5, Cm, "mk,kn->mn", 2.0, A, B)
    assert np.max(np.abs(Cm - (0.5 * C0 + 2.0 * A @ B))) < 1e-12


def test_contract_strided_views(ddla):
    from ddla_gb300 import einsum
    r = rng(6)
    big = uniform(r, (40, 60))
    A = big[::2, ::3]
    B = uniform(r, (20, 12)).T.copy().T        # column-major
    Cm = np.zeros((20, 12))
    einsum.Contract(Cm, "mk,kn->mn", 1.0, A, B)
    assert np.max(np.abs(Cm - A @ B)) < 1e-12
