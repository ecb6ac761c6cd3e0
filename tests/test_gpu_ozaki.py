"""GPU: the split-slice (Ozaki) FP64 GEMM on the BF16 tensor cores, against
FP64 references.

Bars:
  * integer operands (|a|, |b| <= 127, products exact in FP64): bit-exact;
  * general operands: |C - C_ref| <= 2^-53 k (4 |alpha| s_i t_j + |alpha| (|A||B|)_ij)
    + 2^-52 |beta C|, with s_i = max_l |a_il| and t_j = max_l |b_lj| (the
    scheme's bound relative to the row / column scales, plus the FP64
    reference's own rounding);
  * factorizations whose trailing updates run on it: backward error <= 1e-14.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import berr, rng

pytestmark = pytest.mark.gpu
U = 2.0 ** -53


def _gemm(ddla, A, B, Cm, alpha, beta, ta=0, tb=0, prec=None):
    import torch
    from ddla_gb300 import device
    a, b, c = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (A, B, Cm))
    h = device.Handle(torch.cuda.current_stream())
    h.gemm(alpha, a, b, beta, c, ta=ta, tb=tb, precision=ddla.PREC_OZAKI if prec is None else prec)
    h.sync()
    out = c.cpu().numpy()
    h.close()
    return out


def _bound(A, B, Cm, alpha, beta):
    k = A.shape[1]
    s = np.abs(A).max(axis=1, initial=0.0)[:, None]
    t = np.abs(B).max(axis=0, initial=0.0)[None, :]
    return U * k * (4 * abs(alpha) * s * t + abs(alpha) * (np.abs(A) @ np.abs(B))) + 2 * U * abs(beta) * np.abs(Cm)


SHAPES = [(1, 1, 1), (37, 45, 70), (128, 32, 64), (129, 33, 65), (300, 257, 1000), (256, 96, 4100), (64, 700, 200)]


@pytest.mark.parametrize("m,n,k", SHAPES)
def test_ozaki_accuracy(ddla, m, n, k):
    r = rng(m * 31 + n * 7 + k)
    A, B, Cm = r.standard_normal((m, k)), r.standard_normal((k, n)), r.standard_normal((m, n))
    out = _gemm(ddla, A, B, Cm, -1.0, 1.0)
    ref = -(A @ B) + Cm
    assert np.all(np.abs(out - ref) <= _bound(A, B, Cm, -1.0, 1.0))


def test_ozaki_integers_bit_exact(ddla):
    # slices hold every bit of 8-bit integers and every level accumulates
    # exactly, so the product is exact (k spans several flush periods)
    r = rng(77)
    for (m, n, k) in [(200, 70, 1500), (130, 40, 5000)]:
        A = r.integers(-127, 128, (m, k)).astype(np.float64)
        B = r.integers(-127, 128, (k, n)).astype(np.float64)
        exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
        out = _gemm(ddla, A, B, np.zeros((m, n)), 1.0, 0.0)
        assert np.array_equal(out, exact)


def test_ozaki_dynamic_range(ddla):
    # rows / columns spread over 2^-40 .. 2^40: the error scales with each
    # row's and column's own magnitude
    r = rng(78)
    m, n, k = 160, 90, 700
    A = r.standard_normal((m, k)) * np.exp2(r.integers(-40, 41, (m, 1)))
    B = r.standard_normal((k, n)) * np.exp2(r.integers(-40, 41, (1, n)))
    A[3, :] = 0.0
    out = _gemm(ddla, A, B, np.zeros((m, n)), 1.0, 0.0)
    ref = A @ B
    assert np.all(out[3] == 0.0)
    assert np.all(np.abs(out - ref) <= _bound(A, B, np.zeros((m, n)), 1.0, 0.0))


def test_ozaki_subnormal_row(ddla):
    # a row of subnormals keeps its own scale; the result row is subnormal, so
    # the reference and the product differ by at most a few subnormal ulps
    r = rng(85)
    A, B = r.standard_normal((20, 64)), r.standard_normal((64, 24))
    A[5] = r.standard_normal(64) * 1e-310
    out = _gemm(ddla, A, B, np.zeros((20, 24)), 1.0, 0.0)
    ref = A @ B
    tiny = 2.0 ** -1074
    assert np.all(np.abs(out - ref) <= _bound(A, B, np.zeros((20, 24)), 1.0, 0.0) + 64 * tiny)
    assert np.any(out[5] != 0.0)


def test_ozaki_transposes_alpha_beta(ddla):
    r = rng(79)
    m, n, k = 150, 70, 300
    At, Bt = r.standard_normal((k, m)), r.standard_normal((n, k))
    Cm = r.standard_normal((m, n))
    out = _gemm(ddla, At, Bt, Cm, 0.75, -2.0, ta=ddla.TRANSPOSE, tb=ddla.TRANSPOSE)
    ref = 0.75 * (At.T @ Bt.T) - 2.0 * Cm
    assert np.all(np.abs(out - ref) <= _bound(At.T, Bt.T, Cm, 0.75, -2.0))
    # alpha = 0 and k = 0 give beta * C
    out0 = _gemm(ddla, At, Bt, Cm, 0.0, 0.5, ta=ddla.TRANSPOSE, tb=ddla.TRANSPOSE)
    assert np.array_equal(out0, 0.5 * Cm)
    outk = _gemm(ddla, np.zeros((m, 0)), np.zeros((0, n)), Cm, 1.0, 3.0)
    assert np.array_equal(outk, 3.0 * Cm)


def test_ozaki_nonfinite_row(ddla):
    r = rng(80)
    A, B = r.standard_normal((40, 50)), r.standard_normal((50, 30))
    A[7, 3] = np.inf
    out = _gemm(ddla, A, B, np.zeros((40, 30)), 1.0, 0.0)
    assert not np.isfinite(out[7]).any()
    keep = np.arange(40) != 7
    assert np.all(np.abs(out[keep] - (A @ B)[keep]) <= _bound(A[keep], B, np.zeros((39, 30)), 1.0, 0.0))


def test_ozaki_matches_dmma_closely(ddla):
    # both paths are FP64-accurate: their difference is at the FP64 rounding level
    r = rng(81)
    A, B = r.uniform(-1, 1, (512, 2048)), r.uniform(-1, 1, (2048, 384))
    oz = _gemm(ddla, A, B, np.zeros((512, 384)), 1.0, 0.0)
    dm = _gemm(ddla, A, B, np.zeros((512, 384)), 1.0, 0.0, prec=ddla.PREC_FP64)
    scale = np.abs(A) @ np.abs(B)
    assert np.max(np.abs(oz - dm) / scale) <= 64 * U


def test_lu_with_ozaki_updates(ddla):
    import torch
    from ddla_gb300 import device
    r = rng(82)
    n = 1500
    A = r.standard_normal((n, n))
    b = r.standard_normal((n, 2))
    a = torch.from_numpy(A.copy()).cuda()
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    h = device.Handle(torch.cuda.current_stream())
    assert h.getrf(a, piv, precision=ddla.PREC_OZAKI) == 0
    x = torch.from_numpy(b.copy()).cuda()
    h.getrs(a, piv, x)
    h.sync()
    X = x.cpu().numpy()
    h.close()
    assert berr(A, X, b) <= 1e-14


def test_cholesky_with_ozaki_updates(ddla):
    import torch
    from ddla_gb300 import device
    from helpers import spd
    r = rng(83)
    n = 1100
    A = spd(r, n)
    b = r.standard_normal((n, 1))
    for uplo in (ddla.LOWER, ddla.UPPER):
        a = torch.from_numpy(A.copy()).cuda()
        h = device.Handle(torch.cuda.current_stream())
        assert h.potrf(uplo, a, precision=ddla.PREC_OZAKI) == 0
        x = torch.from_numpy(b.copy()).cuda()
        h.potrs(uplo, a, x)
        h.sync()
        X = x.cpu().numpy()
        h.close()
        assert berr(A, X, b) <= 1e-14


def test_einsum_ozaki_precision(ddla):
    from ddla_gb300 import einsum
    r = rng(84)
    L = r.standard_normal((6, 40, 50))
    R = r.standard_normal((50, 6, 30))
    out64 = np.zeros((6, 40, 30))
    outoz = np.zeros((6, 40, 30))
    einsum.Contract(out64, "bik,kbj->bij", 1.0, L, R)
    einsum.Contract(outoz, "bik,kbj->bij", 1.0, L, R, precision=ddla.PREC_OZAKI)
    ref = np.einsum("bik,kbj->bij", L, R)
    scale = np.einsum("bik,kbj->bij", np.abs(L), np.abs(R))
    assert np.max(np.abs(out64 - ref) / scale) <= 64 * U
    assert np.max(np.abs(outoz - ref) / scale) <= 256 * U
