"""Multi-operand einsum (MArray.Einsum, DDLA/Einsum/MArray.Contract.cs:409-427)
with DDLA's greedy pairwise path (EinsumTree/EinsumState.cs:45-419).

CPU: the oracle's restatement of the path against numpy.einsum, and the
library's path (C ABI, no GPU needed) identical to the oracle's.  The GPU
tests are in test_gpu_einsum_multi.py."""
import numpy as np
import pytest

from helpers import rng, uniform

CASES = [
    ("ab,bc,cd->ad", [(10, 20), (20, 30), (30, 5)]),
    ("ij,jk,kl,lm->im", [(4, 8), (8, 16), (16, 2), (2, 64)]),
    ("abc,cd,de,bf->aef", [(2, 3, 4), (4, 5), (5, 6), (3, 7)]),
    ("ij,jk,ki->", [(6, 7), (7, 8), (8, 6)]),
    ("bik,bkj,bjl->bil", [(3, 5, 6), (3, 6, 7), (3, 7, 4)]),
    ("ab,cd,bc->ad", [(9, 9), (9, 9), (9, 9)]),          # equal costs: ties to the smaller l, then r
    ("i,i,i->i", [(11,), (11,), (11,)]),
    ("ijk,jl,kl,lm->im", [(3, 4, 5), (4, 6), (5, 6), (6, 2)]),
]


@pytest.mark.parametrize("expr,shapes", CASES)
def test_oracle_einsum_matches_numpy(orc, expr, shapes):
    r = rng(60 + len(expr))
    ops = [uniform(r, s) for s in shapes]
    got = orc.einsum(expr, ops)
    ref = np.einsum(expr, *ops)
    assert np.max(np.abs(got - ref)) <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("expr,shapes", CASES)
def test_library_path_matches_oracle(ddla, orc, expr, shapes):
    from ddla_gb300 import einsum as es
    assert es.einsum_path(expr, *shapes) == orc.einsum_path(expr, shapes)


def test_path_tie_and_quirk(orc):
    # (0,2) -> "ac" and (1,2) -> "bd" both cost 81 and (0,1) -> "abcd" 6561:
    # the tie goes to the smaller l
    assert orc.einsum_path("ab,cd,bc->ad", [(9, 9)] * 3) == ["ab,bc->ac", "ac,cd->ad"]
    # inputs count as size 0 but intermediates with their size: after
    # (0,1) -> "ac" (4, tied with "cd,de->ce"), "ac,cd->ad" costs 4 - 4 = 0,
    # below "cd,de->ce" (4) and "ac,de->acde" (16 - 4)
    assert orc.einsum_path("ab,bc,cd,de->ae", [(2, 50), (50, 2), (2, 2), (2, 2)]) == \
        ["ab,bc->ac", "ac,cd->ad", "ad,de->ae"]
    # with d = 50 the intermediate-free pair wins the second step
    assert orc.einsum_path("ab,bc,cd,de->ae", [(2, 50), (50, 2), (2, 50), (50, 2)]) == \
        ["ab,bc->ac", "cd,de->ce", "ac,ce->ae"]


def test_path_errors(ddla):
    from ddla_gb300 import einsum as es
    with pytest.raises(Exception):
        es.einsum_path("ab,bc->ad", (2, 3), (3, 4))          # target symbol missing from the inputs
    with pytest.raises(Exception):
        es.einsum_path("ab,bc->ac", (2, 3), (4, 4))          # conflicting lengths
