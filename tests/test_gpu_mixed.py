"""Mixed-precision solves: FP32 factorization + FP64 refinement reach the
FP64 backward-error target and agree with the FP64 oracle solution."""
import numpy as np
import pytest

from helpers import berr, rng, spd

pytestmark = pytest.mark.gpu


# n = 1001 and 2050: rows not 16-byte aligned (the element-wise form of the
# fused next-panel step) and a last panel narrower than 64
@pytest.mark.parametrize("prec", ["fp32", "tf32x3", "bf16x3"])
@pytest.mark.parametrize("n,nrhs", [(100, 1), (1001, 1), (1024, 1), (2048, 4), (2050, 2), (3000, 16)])
def test_mixed_lu_reaches_fp64(ddla, orc, n, nrhs, prec):
    r = rng(n)
    A = r.standard_normal((n, n))
    B = r.standard_normal((n, nrhs))
    F = A.copy()
    info, piv = orc.dgetrf(F)
    Xo = B.copy()
    orc.dgetrs(F, piv, Xo)
    X, rep = ddla.solve_mixed(A, B, precision=getattr(ddla, "PREC_" + prec.upper()), x_ref=Xo)
    assert rep["converged"] == 1
    assert rep["backward_error"] <= 1e-14
    assert berr(A, X, B) <= 1e-14
    assert rep["forward_error"] <= 1e-10


@pytest.mark.parametrize("prec", ["fp32", "tf32x3", "bf16x3"])
@pytest.mark.parametrize("n,nrhs", [(500, 16), (2048, 16)])
def test_mixed_cholesky(ddla, orc, n, nrhs, prec):
    r = rng(n + 1)
    A = spd(r, n)
    B = r.standard_normal((n, nrhs))
    X, rep = ddla.solve_mixed(A, B, spd=True, precision=getattr(ddla, "PREC_" + prec.upper()))
    assert rep["converged"] == 1 and rep["backward_error"] <= 1e-14
    assert berr(A, X, B) <= 1e-14


def test_mixed_no_refinement_reports_not_converged(ddla):
    r = rng(1)
    A = r.standard_normal((300, 300))
    B = r.standard_normal((300, 1))
    with pytest.raises(ddla.DDLAError) as e:
        ddla.solve_mixed(A, B, precision=ddla.PREC_FP32, max_iter=-1)
    assert e.value.code == -1004


def test_gmres_refinement_on_ill_conditioned(ddla):
    # kappa ~ 1e7 or more: classical refinement contracts slowly or not at
    # all, GMRES-IR (the default for one right-hand side) reaches the FP64
    # backward-error target
    from ddla_gb300 import autotune
    from helpers import berr, rng
    r = rng(321)
    n = 1024
    A = r.standard_normal((n, n))
    U, sv, Vt = np.linalg.svd(A)
    A = A - (sv[-1] - sv[-1] / 3e3) * np.outer(U[:, -1], Vt[-1])
    b = r.standard_normal((n, 1))
    x, rep = ddla.solve_mixed(A, b)
    assert rep["converged"] and berr(A, x, b) <= 1e-14
    # classical refinement: slower, or no convergence at all at this kappa
    try:
        autotune.tune_set("refine.gmres", 0)
        x2, rep2 = ddla.solve_mixed(A, b, max_iter=80)
        assert rep["iterations"] <= rep2["iterations"]
    except ddla.DDLAError as e:
        assert e.code == ddla._lib.ERR_NOT_CONVERGED
    finally:
        autotune.tune_set("refine.gmres", 1)


def _growth_of(kind, F, A):
    """The report's growth figures from an FP64 factor (oracle): LU
    max|U|/max|A| and the U diagonal ratio; Cholesky max_i sum_k l_ik^2 /
    max|A| and the ratio of l_ii^2; LDL^T max_i (sum_k<i l_ik^2 |d_k| + |d_i|) /
    max|A| and the ratio of |d_i|."""
    amax = np.abs(A).max()
    if kind == "lu":
        U = np.triu(F)
        d = np.abs(np.diag(F))
        return np.abs(U).max() / amax, d.max() / d.min()
    L = np.tril(F)
    if kind == "chol":
        d = np.diag(F) ** 2
        return (L * L).sum(1).max() / amax, d.max() / d.min()
    d = np.abs(np.diag(F))
    Ls = np.tril(F, -1)
    return ((Ls * Ls) @ d + d).max() / amax, d.max() / d.min()


def _sym_indefinite(r, n):
    # symmetric, indefinite, leading blocks far from singular: the unpivoted
    # LDL^T of DDLA's LDLT applies
    S = r.standard_normal((n, n))
    S = (S + S.T) / 2
    return S + np.diag(np.where(np.arange(n) % 3 == 0, -1.0, 1.0) * 2.0 * np.sqrt(n))


@pytest.mark.parametrize("prec", ["fp32", "tf32x3", "bf16x3"])
@pytest.mark.parametrize("n,nrhs,kind", [(300, 1, "spd"), (2048, 4, "spd"), (1500, 3, "indef"), (3000, 16, "indef")])
def test_mixed_ldlt_reaches_fp64(ddla, orc, n, nrhs, kind, prec):
    r = rng(n + nrhs)
    A = spd(r, n) if kind == "spd" else _sym_indefinite(r, n)
    B = r.standard_normal((n, nrhs))
    F = A.copy()
    assert orc.dldlt(ddla.LOWER, F) == 0
    Xo = B.copy()
    orc.dldlts(ddla.LOWER, F, Xo)
    X, rep = ddla.solve_mixed(A, B, ldlt=True, precision=getattr(ddla, "PREC_" + prec.upper()), x_ref=Xo)
    assert rep["converged"] == 1 and rep["backward_error"] <= 1e-14
    assert berr(A, X, B) <= 1e-14
    assert rep["forward_error"] <= 1e-10
    g, dr = _growth_of("ldlt", F, A)
    assert abs(rep["growth"] - g) <= 1e-3 * g
    assert abs(rep["diag_ratio"] - dr) <= 1e-3 * dr


@pytest.mark.parametrize("kind", ["lu", "chol"])
def test_growth_monitor_matches_fp64_factor(ddla, orc, kind):
    n = 1200
    r = rng(4321)
    A = spd(r, n) if kind == "chol" else r.standard_normal((n, n))
    B = r.standard_normal((n, 1))
    F = A.copy()
    if kind == "lu":
        info, piv = orc.dgetrf(F)
    else:
        info = orc.dpotrf(ddla.LOWER, F)
    assert info == 0
    X, rep = ddla.solve_mixed(A, B, spd=kind == "chol")
    g, dr = _growth_of(kind, F, A)
    # FP32 factors of the same matrix; LU may pivot differently after a near-tie
    tol = 1e-3 if kind == "chol" else 0.25
    assert abs(rep["growth"] - g) <= tol * g, (rep["growth"], g)
    assert rep["diag_ratio"] >= 1.0


@pytest.mark.parametrize("mode", ["lu", "chol", "ldlt"])
def test_mixed_more_than_16_rhs(ddla, orc, mode):
    # DDLA's Cholesky tests solve 256 right-hand sides
    # (Tests/TestFlame/TestChol.cs:101-162); the mixed solvers refine them in
    # blocks of 16 with one factorization
    n, nrhs = 700, 41
    r = rng(99)
    A = spd(r, n) if mode != "lu" else r.standard_normal((n, n))
    B = r.standard_normal((n, nrhs))
    X, rep = ddla.solve_mixed(A, B, spd=mode == "chol", ldlt=mode == "ldlt")
    assert rep["converged"] == 1
    assert berr(A, X, B) <= 1e-14
    assert np.max(np.abs(X - np.linalg.solve(A, B))) / np.abs(X).max() <= 1e-10
