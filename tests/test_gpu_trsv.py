"""GPU: single-right-hand-side triangular solves, the cluster solve (one
thread-block cluster, x exchanged over DSMEM) against the chained per-block
solve and the oracle, for both triangles, unit / non-unit diagonals,
transposes, sizes off the 64-row block and off the 16-byte row alignment."""
import numpy as np
import pytest

from helpers import rel_max, rng

pytestmark = pytest.mark.gpu


def _tri(r, n, lower, unit):
    A = r.uniform(-1, 1, (n, n)) / n
    A += np.eye(n) * (1.0 if unit else 2.0)
    return np.tril(A) if lower else np.triu(A)


@pytest.mark.parametrize("n", [65, 130, 257, 1000, 2051, 4096])
@pytest.mark.parametrize("uplo", ["L", "U"])
def test_cluster_vs_chain_vs_oracle(ddla, orc, n, uplo):
    from ddla_gb300 import autotune
    r = rng(n * 3 + (uplo == "U"))
    lower = uplo == "L"
    for trans in (ddla.NO_TRANSPOSE, ddla.TRANSPOSE):
        for unit in (False, True):
            A = _tri(r, n, lower, unit)
            b = r.standard_normal((n, 1))
            u = ddla.LOWER if lower else ddla.UPPER
            d = ddla.UNIT if unit else ddla.NONUNIT
            xo = b.copy()
            orc.dtrsm(orc.LEFT, u, trans, d, 1.0, A, xo)
            xc = b.copy()
            ddla.BlasProvider.TrSM(ddla.LEFT, u, trans, d, 1.0, A, xc)
            try:
                autotune.tune_set("trsv.cluster", 0)
                xs = b.copy()
                ddla.BlasProvider.TrSM(ddla.LEFT, u, trans, d, 1.0, A, xs)
            finally:
                autotune.tune_set("trsv.cluster", 1)
            assert rel_max(xc, xo) <= 1e-12
            assert rel_max(xs, xo) <= 1e-12


def test_cluster_solve_in_mixed_refinement(ddla):
    # n not a multiple of 4: the FP32 factor rows are not 16-byte aligned, so
    # the tiles go through the element-wise copy path
    from helpers import berr
    r = rng(77)
    for n in (1023, 3001):
        A = r.standard_normal((n, n))
        b = r.standard_normal((n, 1))
        x, rep = ddla.solve_mixed(A, b)
        assert rep["converged"] and berr(A, x, b) <= 1e-14


@pytest.mark.parametrize("n", [64, 200, 1000, 2051])
@pytest.mark.parametrize("nrhs", [9, 13, 16])
def test_chain16_vs_chain_vs_oracle(ddla, orc, n, nrhs):
    # 9-16 right-hand sides: the 16-wide chained solve (one thread per row and
    # right-hand side, tiles by 16-byte copies; n = 2051 has unaligned rows and
    # keeps the 4-group chain) against the 4-group chain and the oracle, both
    # triangles, both transposes (the transposed views stream column tiles)
    from ddla_gb300 import autotune
    r = rng(n * 5 + nrhs)
    for lower in (True, False):
        for trans in (ddla.NO_TRANSPOSE, ddla.TRANSPOSE):
            for unit in (False, True):
                A = _tri(r, n, lower, unit)
                B = r.standard_normal((n, nrhs))
                u = ddla.LOWER if lower else ddla.UPPER
                d = ddla.UNIT if unit else ddla.NONUNIT
                xo = B.copy()
                orc.dtrsm(orc.LEFT, u, trans, d, 1.0, A, xo)
                x16 = B.copy()
                ddla.BlasProvider.TrSM(ddla.LEFT, u, trans, d, 1.0, A, x16)
                try:
                    autotune.tune_set("trsv.chain16", 0)
                    x4 = B.copy()
                    ddla.BlasProvider.TrSM(ddla.LEFT, u, trans, d, 1.0, A, x4)
                finally:
                    autotune.tune_set("trsv.chain16", 1)
                assert rel_max(x16, xo) <= 1e-12
                assert rel_max(x4, xo) <= 1e-12
