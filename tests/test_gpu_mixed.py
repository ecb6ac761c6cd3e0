"""Mixed-precision solves: FP32 factorization + FP64 refinement reach the
FP64 backward-error target and agree with the FP64 oracle solution."""
import numpy as np
import pytest

from helpers import berr, rng, spd

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp32", "tf32x3", "bf16x3"])
@pytest.mark.parametrize("n,nrhs", [(100, 1), (1024, 1), (2048, 4), (3000, 16)])
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
