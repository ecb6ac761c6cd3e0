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
