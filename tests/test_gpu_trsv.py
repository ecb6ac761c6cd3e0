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


_SPLIT_DEFAULTS = {"trsv.split.w": 16, "trsv.split.pw": 6, "trsv.split.clusters": 0, "trsv.fused": 1}


def _with_tune(setting, fn):
    from ddla_gb300 import autotune
    try:
        for k, v in setting.items():
            autotune.tune_set(k, v)
        return fn()
    finally:
        for k in setting:
            autotune.tune_set(k, _SPLIT_DEFAULTS[k])


@pytest.mark.parametrize("n", [1500, 2051, 4096])
@pytest.mark.parametrize("setting", [{}, {"trsv.split.w": 4, "trsv.split.pw": 2}, {"trsv.split.clusters": 2},
                                     {"trsv.split.w": 24, "trsv.split.pw": 24}, {"trsv.fused": 0},
                                     {"trsv.fused": 0, "trsv.split.pw": 1}])
def test_split_solve_vs_oracle(ddla, orc, n, setting):
    """One right-hand side through the split solve: the chain cluster on the
    tiles near the diagonal, helper clusters summing the far tiles.  Narrow
    and wide near windows; with one helper cluster (clusters = 2) the chain
    finds most rows untaken and sums them itself; without the last-tile
    products (trsv.fused = 0) every block takes its last tile and its inverse
    after the previous x.  Against the oracle and the one-cluster solve
    (trsv.split.w = 0); n = 2051 has unaligned rows (element copies), n = 1500
    few far rows."""
    r = rng(n * 7 + len(setting))
    for lower in (True, False):
        for trans in (ddla.NO_TRANSPOSE, ddla.TRANSPOSE):
            unit = trans == ddla.TRANSPOSE
            A = _tri(r, n, lower, unit)
            b = r.standard_normal((n, 1))
            u = ddla.LOWER if lower else ddla.UPPER
            d = ddla.UNIT if unit else ddla.NONUNIT
            xo = b.copy()
            orc.dtrsm(orc.LEFT, u, trans, d, 1.0, A, xo)

            def run():
                x = b.copy()
                ddla.BlasProvider.TrSM(ddla.LEFT, u, trans, d, 1.0, A, x)
                return x
            xs = _with_tune(setting, run)
            x1 = _with_tune({"trsv.split.w": 0}, run)
            assert rel_max(xs, xo) <= 1e-12
            assert rel_max(xs, x1) <= 1e-12


@pytest.mark.parametrize("n", [3001, 4096])
def test_split_solve_in_mixed_refinement(ddla, n):
    """The FP32 correction solves of the mixed LU solve through the split
    solve (with and without the last-tile products, with few helpers): the
    same solution and the same number of preconditioner applications (within
    one) as with the one-cluster solve."""
    from helpers import berr
    r = rng(n + 11)
    A = r.standard_normal((n, n))
    b = r.standard_normal((n, 1))
    xs, reps = _with_tune({}, lambda: ddla.solve_mixed(A, b))
    x1, rep1 = _with_tune({"trsv.split.w": 0}, lambda: ddla.solve_mixed(A, b))
    xc, repc = _with_tune({"trsv.split.clusters": 2}, lambda: ddla.solve_mixed(A, b))
    xf, repf = _with_tune({"trsv.fused": 0}, lambda: ddla.solve_mixed(A, b))
    for x, rep in ((xs, reps), (x1, rep1), (xc, repc), (xf, repf)):
        assert rep["converged"] and berr(A, x, b) <= 1e-14
    for rep in (reps, repc, repf):
        assert abs(rep["iterations"] - rep1["iterations"]) <= 1
    assert rel_max(xs, x1) <= 1e-12
