"""GPU: the tcgen05 3xTF32 GEMM (trailing updates of the mixed factorizations)
against an FP64 reference.  3xTF32 products carry ~2^-21 relative error per
term; the bar is max|C - C_ref| <= 2e-5 * (|alpha| |A| |B| + |beta| |C|)
elementwise-normalised, i.e. FP32-level accuracy."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(128, 64, 64), (300, 200, 64), (129, 65, 8), (257, 130, 100), (64, 64, 1), (1000, 1000, 64),
          (512, 768, 256), (33, 17, 64)]


def _run(ddla, prec, m, n, k, alpha, beta, seed):
    import torch
    from ddla_gb300 import device
    g = torch.Generator().manual_seed(seed)
    A = torch.rand(m, k, generator=g, dtype=torch.float64) * 2 - 1
    B = torch.rand(k, n, generator=g, dtype=torch.float64) * 2 - 1
    Cm = torch.rand(m, n, generator=g, dtype=torch.float64) * 2 - 1
    ref = (alpha * A.numpy() @ B.numpy() + beta * Cm.numpy())
    scale = abs(alpha) * (np.abs(A.numpy()) @ np.abs(B.numpy())) + abs(beta) * np.abs(Cm.numpy())
    a, b, c = A.float().cuda(), B.float().cuda(), Cm.float().cuda()
    h = device.Handle(torch.cuda.current_stream())
    rc = ddla.lib().ddla_dev_sgemm_tc(h.h, prec, m, n, k, alpha, C.c_void_p(a.data_ptr()), k, 1,
                                      C.c_void_p(b.data_ptr()), n, 1, beta, C.c_void_p(c.data_ptr()), n, 1)
    ddla._lib.check(rc, "sgemm_tc")
    h.sync()
    out = c.double().cpu().numpy()
    h.close()
    return np.max(np.abs(out - ref) / scale)


@pytest.mark.parametrize("m,n,k", SHAPES)
def test_tf32x3_accuracy(ddla, m, n, k):
    err = _run(ddla, ddla.PREC_TF32X3, m, n, k, -1.0, 1.0, m * 7 + n)
    assert err <= 2e-5, err


def test_tf32x3_alpha_beta(ddla):
    assert _run(ddla, ddla.PREC_TF32X3, 200, 100, 64, 0.5, 0.0, 3) <= 2e-5
    assert _run(ddla, ddla.PREC_TF32X3, 200, 100, 64, 2.0, -0.5, 4) <= 2e-5


def test_fp32_reference_path(ddla):
    assert _run(ddla, ddla.PREC_FP32, 300, 200, 64, -1.0, 1.0, 5) <= 2e-6


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (300, 200, 64), (129, 257, 17), (1000, 900, 64), (64, 1, 64),
                                   (2000, 4100, 64), (1, 300, 8)])
def test_tf32x3_rank_update_path(ddla, m, n, k):
    # beta = 1 and k <= 64: the packed-operand persistent update kernel
    err = _run(ddla, ddla.PREC_TF32X3, m, n, k, -1.0, 1.0, m + 3 * n + k)
    assert err <= 2e-5, err


@pytest.mark.parametrize("n,k", [(128, 64), (300, 64), (515, 40), (1000, 64), (257, 8)])
def test_tf32x3_update_transposed_b(ddla, n, k):
    # C (n x n) += -A A^T with B = A^T given as a transposed view (rs = 1,
    # cs = k): the shape of the Cholesky trailing update
    import torch
    from ddla_gb300 import device
    g = torch.Generator().manual_seed(n + k)
    A = torch.rand(n, k, generator=g, dtype=torch.float64) * 2 - 1
    Cm = torch.rand(n, n, generator=g, dtype=torch.float64) * 2 - 1
    ref = Cm.numpy() - A.numpy() @ A.numpy().T
    scale = np.abs(A.numpy()) @ np.abs(A.numpy().T) + np.abs(Cm.numpy())
    a, c = A.float().cuda(), Cm.float().cuda()
    h = device.Handle(torch.cuda.current_stream())
    rc = ddla.lib().ddla_dev_sgemm_tc(h.h, ddla.PREC_TF32X3, n, n, k, -1.0, C.c_void_p(a.data_ptr()), k, 1,
                                      C.c_void_p(a.data_ptr()), 1, k, 1.0, C.c_void_p(c.data_ptr()), n, 1)
    ddla._lib.check(rc, "sgemm_tc")
    h.sync()
    out = c.double().cpu().numpy()
    h.close()
    assert np.max(np.abs(out - ref) / scale) <= 2e-5


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (300, 200, 64), (129, 257, 17), (1000, 900, 64), (64, 1, 64),
                                   (2000, 4100, 64), (1, 300, 8), (515, 515, 40)])
def test_bf16x3_rank_update_path(ddla, m, n, k):
    # 3xBF16: x = hi + lo with two bf16 parts (16 significant bits), products
    # hi*hi + hi*lo + lo*hi, FP32 accumulation: about 2^-16 relative to
    # |A||B| per element.  n not a multiple of 4 takes the scalar C path.
    err = _run(ddla, ddla.PREC_BF16X3, m, n, k, -1.0, 1.0, 11 * m + n + k)
    assert err <= 5e-5, err


def test_bf16x3_only_as_rank_update(ddla):
    # beta != 1 or k > 64 is not the update shape: a clear unsupported status
    import torch
    from ddla_gb300 import device
    a = torch.zeros(64, 128, dtype=torch.float32, device="cuda")
    h = device.Handle(torch.cuda.current_stream())
    rc = ddla.lib().ddla_dev_sgemm_tc(h.h, ddla.PREC_BF16X3, 64, 64, 128, -1.0, C.c_void_p(a.data_ptr()), 128, 1,
                                      C.c_void_p(a.data_ptr()), 64, 1, 1.0, C.c_void_p(a.data_ptr()), 64, 1)
    h.close()
    assert rc == ddla._lib.ERR_UNSUPPORTED


def test_bf16x3_update_column_major_c(ddla):
    # C given as a transposed (column-major) view: column stride != 1
    import torch
    from ddla_gb300 import device
    m, n, k = 300, 260, 64
    g = torch.Generator().manual_seed(9)
    A = torch.rand(m, k, generator=g, dtype=torch.float64) * 2 - 1
    B = torch.rand(k, n, generator=g, dtype=torch.float64) * 2 - 1
    Cm = torch.rand(m, n, generator=g, dtype=torch.float64) * 2 - 1
    ref = Cm.numpy() - A.numpy() @ B.numpy()
    scale = np.abs(A.numpy()) @ np.abs(B.numpy()) + np.abs(Cm.numpy())
    a, b = A.float().cuda(), B.float().cuda()
    ct = Cm.float().T.contiguous().cuda()          # n x m storage: C(i, j) at j * m + i
    h = device.Handle(torch.cuda.current_stream())
    rc = ddla.lib().ddla_dev_sgemm_tc(h.h, ddla.PREC_BF16X3, m, n, k, -1.0, C.c_void_p(a.data_ptr()), k, 1,
                                      C.c_void_p(b.data_ptr()), n, 1, 1.0, C.c_void_p(ct.data_ptr()), 1, m)
    ddla._lib.check(rc, "sgemm_tc")
    h.sync()
    out = ct.double().cpu().numpy().T
    h.close()
    assert np.max(np.abs(out - ref) / scale) <= 5e-5
