"""CPU: the product's einsum index analysis (ddla_contract_plan, host code of
the C ABI) equals the oracle's restatement of MArray.Contract's analysis."""
import numpy as np
import pytest

CASES = [
    ("mnk,nktc->mct", (5, 7, 9), (7, 9, 4, 3), (5, 3, 4)),
    ("mk,kn->mn", (37, 29), (29, 23), (37, 23)),
    ("bik,bkj->bij", (6, 20, 21), (6, 21, 22), (6, 20, 22)),
    ("abcd,cdef->abef", (4, 5, 6, 7), (6, 7, 3, 2), (4, 5, 3, 2)),
    ("ij,jk->ki", (11, 13), (13, 17), (17, 11)),
    ("aij,ajk->ik", (3, 8, 9), (3, 9, 10), (8, 10)),
    ("ii,ij->j", (6, 6), (6, 5), (5,)),
    ("abc,c->ab", (3, 4, 5), (5,), (3, 4)),
]


@pytest.mark.parametrize("expr,sa,sb,sc", CASES)
def test_plan_matches_oracle(ddla, orc, expr, sa, sb, sc):
    from ddla_gb300 import einsum
    A, B, Cm = np.zeros(sa), np.zeros(sb), np.zeros(sc)
    got = einsum.plan(expr, A, B, Cm).as_dict()
    exp = orc.plan_dict(orc.contract_plan(expr, A, B, Cm))
    assert got == exp


def test_plan_rejects_bad_expression(ddla):
    from ddla_gb300 import einsum
    with pytest.raises(ValueError):
        einsum.plan("ab,bc", np.zeros((2, 2)), np.zeros((2, 2)), np.zeros((2, 2)))
    with pytest.raises(ValueError):
        einsum.plan("ab,bc->ac", np.zeros((2, 3)), np.zeros((4, 2)), np.zeros((2, 2)))
