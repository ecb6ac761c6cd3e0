"""GPU parity at the benchmark configurations' own sizes.

The other GPU test files compare the CUDA path with the oracle on many small
and medium cases; these run each configuration the benchmark measures at its
full size, on the same kind of seeded inputs:

* LU + solve, n = 8192, N(0,1): the FP64 path's pivot sequence is the
  oracle's (DDLA's PLUDecompose restated, LU.cs:289-374), factors and solution
  agree; the mixed solve reports how far its FP32 factor followed that pivot
  sequence and reaches the FP64 backward-error target.
* SPD Cholesky + solve, n = 16384, G G^T/n + I, 16 right-hand sides: the
  forward error of every mixed precision against the FP64 GPU solve (whose
  Cholesky is pinned to the oracle at n = 4096 here and at n <= 1000 in
  test_gpu_factor.py).
* 20,000 batched solves, n ~ U{8..256}: every item against the oracle.
* einsum 'bik,bkj->bij' (512 x 256^3) and 'abcd,cdef->abef' (64^6): full size
  against the oracle's block-scatter contraction.

The oracle runs on all host cores here (it is the checker; its speed is not
measured in these tests).
"""
import os

import numpy as np
import pytest

from helpers import berr, pivot_tie_ok, rel_max, rng, schur_pivot_gap, spd, uniform

pytestmark = pytest.mark.gpu

HEADLINE_SEED = 0xDD1A0002   # the benchmark's seed for the n = 8192 system


@pytest.fixture(scope="module")
def all_cores(orc):
    orc.set_threads(os.cpu_count() or 1)
    yield
    orc.set_threads(1)


@pytest.fixture(scope="module")
def lu8192(orc, all_cores):
    n = 8192
    r = rng(HEADLINE_SEED)
    A = r.standard_normal((n, n))
    b = r.standard_normal((n, 1))
    Fo = A.copy()
    info, piv_o = orc.dgetrf(Fo)
    assert info == 0
    xo = b.copy()
    orc.dgetrs(Fo, piv_o, xo)
    return A, b, Fo, piv_o, xo


def test_lu_n8192_plain_fp64_matches_oracle(ddla, lu8192):
    A, b, Fo, piv_o, xo = lu8192
    n = A.shape[0]
    Fg = A.copy()
    piv_g = np.zeros(n, dtype=np.int32)
    ddla.LU.PLUDecompose(Fg, piv_g)
    ok, first = pivot_tie_ok(A, piv_g, piv_o)
    assert ok, f"pivot mismatch at {first} that is not a rounding tie"
    if first < 0:
        # same pivot sequence: the factors agree to rounding
        assert rel_max(Fg, Fo) <= 1e-10
    xg = b.copy()
    ddla.LU.PLUSolve(Fg, piv_g, xg)
    assert berr(A, xg, b) <= 1e-14
    assert berr(A, xo, b) <= 1e-14
    # two FP64 solutions of the same system: they differ by ~kappa * u
    assert rel_max(xg, xo) <= 1e-9


@pytest.mark.parametrize("prec", ["tf32x3", "fp32"])
def test_lu_n8192_mixed_reports_pivot_agreement(ddla, lu8192, prec):
    import torch
    from ddla_gb300 import device
    A, b, Fo, piv_o, xo = lu8192
    n = A.shape[0]
    h = device.Handle(torch.cuda.current_stream())
    Ad, bd = torch.from_numpy(A).cuda(), torch.from_numpy(b).cuda()
    X = torch.zeros(n, 1, dtype=torch.float64, device="cuda")
    pref = torch.from_numpy(piv_o.astype(np.int32)).cuda()
    pout = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc, rep = h.gesv_mixed(Ad, bd, X, x_ref=torch.from_numpy(xo).cuda(),
                           precision=getattr(ddla, "PREC_" + prec.upper()), tol=1e-14, piv_ref=pref, piv_out=pout)
    h.sync()
    h.close()
    assert rc == 0 and rep["converged"] == 1
    x = X.cpu().numpy()
    assert berr(A, x, b) <= 1e-14
    # the report's agreement figures are what a direct comparison gives
    p32 = pout.cpu().numpy()
    eq = p32 == piv_o
    assert rep["pivots_agree"] == int(eq.sum())
    diff = np.nonzero(~eq)[0]
    assert rep["pivots_first_diff"] == (int(diff[0]) if diff.size else -1)
    # the FP32 factor follows the FP64 pivot sequence until FP32 rounding
    # flips a near-tie; after that the row orders differ, so agreement of the
    # later entries is incidental.  The first divergence must be such a tie:
    # in the FP64 Schur complement the two candidates differ by a small
    # fraction of the column's largest entry.
    first = rep["pivots_first_diff"]
    if first >= 0:
        assert first >= 64, f"diverged in the first panel (step {first})"
        gap = schur_pivot_gap(A, piv_o, first, p32[first])
        assert gap <= 1e-3, f"pivot at step {first} is not a near-tie (gap {gap:.2e})"
    assert 0 <= rep["forward_error"] <= 1e-9
    assert abs(rep["forward_error"] - rel_max(x, xo)) <= 1e-3 * rep["forward_error"] + 1e-300


def test_cholesky_n4096_plain_fp64_matches_oracle(ddla, orc, all_cores):
    n, nrhs = 4096, 16
    r = rng(0xDD1A0003)
    A = spd(r, n)
    B = r.standard_normal((n, nrhs))
    Fo = A.copy()
    assert orc.dpotrf(0xC0, Fo) == 0
    Fg = A.copy()
    ddla.Cholesky.CholDecompose(ddla.LOWER, Fg)
    assert rel_max(np.tril(Fg), np.tril(Fo)) <= 1e-12
    Xg = ddla.Cholesky(A).Solve(B)
    assert berr(A, Xg, B) <= 1e-14


@pytest.fixture(scope="module")
def chol16384(ddla):
    import torch
    from ddla_gb300 import device
    n, nrhs = 16384, 16
    h = device.Handle(torch.cuda.current_stream())
    g = torch.Generator(device="cuda").manual_seed(0xDD1A0003)
    G = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    A = torch.eye(n, dtype=torch.float64, device="cuda")
    h.gemm(1.0 / n, G, G, 1.0, A, tb=ddla.TRANSPOSE)     # FP64 DMMA: A = G G^T / n + I
    h.sync()
    del G
    A = 0.5 * (A + A.T)
    B = torch.randn(n, nrhs, dtype=torch.float64, device="cuda", generator=g)
    F = A.clone()
    assert h.potrf(ddla.LOWER, F) == 0
    X64 = B.clone()
    h.potrs(ddla.LOWER, F, X64)
    h.sync()
    del F
    torch.cuda.empty_cache()
    yield h, A, B, X64
    h.close()


def _torch_berr(A, X, B):
    R = B - A @ X
    an = A.abs().sum(1).amax()
    return float((R.abs().amax(0) / (an * X.abs().amax(0) + B.abs().amax(0))).max())


def test_cholesky_n16384_plain_fp64_backward_error(chol16384):
    h, A, B, X64 = chol16384
    assert _torch_berr(A, X64, B) <= 1e-14


@pytest.mark.parametrize("prec", ["tf32x3", "fp32", "bf16x3"])
def test_cholesky_n16384_mixed_forward_error(ddla, chol16384, prec):
    import torch
    h, A, B, X64 = chol16384
    X = torch.zeros_like(B)
    rc, rep = h.gesv_mixed(A, B, X, x_ref=X64, precision=getattr(ddla, "PREC_" + prec.upper()), tol=1e-14,
                           spd=True)
    h.sync()
    assert rc == 0 and rep["converged"] == 1, rep
    assert _torch_berr(A, X, B) <= 1e-14
    # kappa(G G^T/n + I) is small, so FP64-level backward error means a
    # forward error near u against the FP64 solve
    fe = float(((X - X64).abs().max() / X64.abs().max()).item())
    assert abs(fe - rep["forward_error"]) <= 1e-3 * fe + 1e-300
    assert fe <= 1e-12


def _batched_items(seed, count):
    r = rng(seed)
    sizes = r.integers(8, 257, count)
    kinds = np.where(np.arange(count) % 2 == 0, 0, 2)
    mats, rhs = [], []
    for nn, k in zip(sizes, kinds):
        if k == 2:
            Gs = r.standard_normal((nn, nn))
            mats.append(Gs @ Gs.T / nn + np.eye(nn))
        else:
            mats.append(r.standard_normal((nn, nn)) + nn * np.eye(nn))
        rhs.append(r.standard_normal(nn))
    return sizes, kinds, mats, rhs


@pytest.fixture(scope="module")
def batched20000(orc, all_cores):
    sizes, kinds, mats, rhs = _batched_items(0xDD1A0004, 20000)
    res_o, info_o = orc.batched(sizes, kinds, mats, rhs)
    assert np.all(info_o == 0)
    return sizes, kinds, mats, rhs, res_o


def test_batched_20000_plain_every_item_matches_oracle(ddla, batched20000):
    import torch
    from ddla_gb300 import batched, device
    sizes, kinds, mats, rhs, res_o = batched20000
    h = device.Handle(torch.cuda.current_stream())
    bs = batched.BatchedSolver(h, sizes, kinds, mixed=False)
    bs.load(mats, rhs)
    bs.run()
    res, info, _ = bs.results()
    bs.close()
    h.close()
    assert np.all(info == 0)
    worst_f = worst_x = worst_b = 0.0
    for i, ((F, x, piv), (Fo, xo, po)) in enumerate(zip(res, res_o)):
        A, b = mats[i], rhs[i]
        if kinds[i] == 0:
            ok, first = pivot_tie_ok(A, piv, po)
            assert ok, f"item {i}: pivot mismatch at {first} that is not a rounding tie"
            if first < 0:
                worst_f = max(worst_f, rel_max(F, Fo))
        else:
            worst_f = max(worst_f, rel_max(np.tril(F), np.tril(Fo)))
        worst_x = max(worst_x, rel_max(x, xo))
        worst_b = max(worst_b, berr(A, x, b))
    assert worst_f <= 1e-10, worst_f
    assert worst_x <= 1e-11, worst_x
    assert worst_b <= 1e-14, worst_b


def test_batched_20000_mixed_every_item_refined(ddla, batched20000):
    import torch
    from ddla_gb300 import batched, device
    sizes, kinds, mats, rhs, res_o = batched20000
    h = device.Handle(torch.cuda.current_stream())
    bs = batched.BatchedSolver(h, sizes, kinds, mixed=True, tol=1e-14)
    bs.load(mats, rhs)
    bs.run()
    res, info, iters = bs.results()
    bs.close()
    h.close()
    assert np.all(info == 0) and np.all(iters >= 0)
    worst_x = worst_b = 0.0
    for i, ((_, x, _), (_, xo, _)) in enumerate(zip(res, res_o)):
        worst_x = max(worst_x, rel_max(x, xo))
        worst_b = max(worst_b, berr(mats[i], x, rhs[i]))
    assert worst_b <= 1e-14, worst_b
    assert worst_x <= 1e-11, worst_x


@pytest.mark.parametrize("expr,shape", [("bik,bkj->bij", (512, 256, 256)), ("abcd,cdef->abef", (64, 64, 64, 64))])
@pytest.mark.parametrize("prec", ["fp64", "ozaki"])
def test_einsum_full_size_matches_oracle(ddla, orc, all_cores, expr, shape, prec):
    from ddla_gb300 import einsum
    r = rng(0xDD1A0005)
    A, B = uniform(r, shape), uniform(r, shape)
    Co = np.zeros(shape)
    orc.contract(expr, 1.0, A, B, Co)
    got = einsum.Contract(expr, 1.0, A, B, precision=getattr(ddla, "PREC_" + prec.upper()))
    # k = 256 or 4096 products of U[-1,1] entries: the oracle's and the GPU's
    # summation orders differ, both are FP64-accurate
    assert np.max(np.abs(got - Co)) / np.abs(Co).max() <= 1e-13
