"""GPU: the allocation-free triangular solve (ddla_dev_dtrsv_noalloc).

It serves callers that must not allocate device memory; its scratch is a
fixed array inside the library, shared by every call.  Checked through the C
ABI against the regular device entry point (ddla_dev_dtrsm, which grows a
handle workspace) on two calls in a row, so the second call runs on scratch
the first one left behind.  This file is collected last so a failure here
cannot hide results of the other GPU tests; it also passes on its own in a
fresh process (it builds everything it needs).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOWER, UPPER, NOTRANS, TRANS, NONUNIT, UNIT, LEFT = 0xC0, 0x60, 0, 8, 0, 0x100, 0


def _case(torch, n, nrhs, seed):
    g = torch.Generator().manual_seed(seed)
    A = (torch.rand(n, n, generator=g, dtype=torch.float64) * 2 - 1) / n + 2 * torch.eye(n, dtype=torch.float64)
    B = torch.rand(n, nrhs, generator=g, dtype=torch.float64) * 2 - 1
    return A.cuda(), B.cuda()


@pytest.mark.parametrize("uplo,trans,diag", [(LOWER, NOTRANS, UNIT), (UPPER, NOTRANS, NONUNIT),
                                             (LOWER, TRANS, NONUNIT), (UPPER, TRANS, UNIT)])
def test_noalloc_matches_regular_solve_twice(ddla, uplo, trans, diag):
    import torch
    from ddla_gb300 import device
    L = ddla.lib()
    stream = torch.cuda.current_stream()
    h = device.Handle(stream)
    for call, (n, nrhs) in enumerate([(1500, 3), (2048, 16)]):
        A, B = _case(torch, n, nrhs, 100 * call + uplo + trans + diag)
        X1 = B.clone()
        rc = L.ddla_dev_dtrsv_noalloc(C.c_void_p(stream.cuda_stream), uplo, trans, diag, n, nrhs,
                                      C.c_void_p(A.data_ptr()), n, 1, C.c_void_p(X1.data_ptr()), nrhs)
        ddla._lib.check(rc, "dtrsv_noalloc")
        X2 = B.clone()
        rc = L.ddla_dev_dtrsm(h.h, LEFT, uplo, trans, diag, n, nrhs, 1.0, C.c_void_p(A.data_ptr()), n, 1,
                              C.c_void_p(X2.data_ptr()), nrhs, 1)
        ddla._lib.check(rc, "dev_dtrsm")
        torch.cuda.synchronize()
        x1, x2 = X1.cpu().numpy(), X2.cpu().numpy()
        assert np.max(np.abs(x1 - x2)) / np.abs(x2).max() <= 1e-12
        # and it really solves the system
        a = A.cpu().numpy()
        T = np.tril(a) if uplo == LOWER else np.triu(a)
        if diag == UNIT:
            np.fill_diagonal(T, 1.0)
        op = T.T if trans == TRANS else T
        assert np.max(np.abs(op @ x1 - B.cpu().numpy())) <= 1e-12
    h.close()


@pytest.mark.parametrize("uplo,trans,diag", [(LOWER, NOTRANS, NONUNIT), (UPPER, TRANS, UNIT)])
def test_noalloc_padded_x_and_strided_a(ddla, uplo, trans, diag):
    # the entry point hands A's strides and X's leading dimension straight to
    # the kernels (no contiguous copy): A a sub-view with row stride 4n and
    # column stride 2 whose gaps hold NaN, X with ldx = nrhs + 3 whose padding
    # must stay untouched; two calls in a row against the handle-based solve on
    # the same views
    import torch
    from ddla_gb300 import device
    L = ddla.lib()
    stream = torch.cuda.current_stream()
    h = device.Handle(stream)
    for call, (n, nrhs) in enumerate([(700, 5), (1029, 16)]):
        A, B = _case(torch, n, nrhs, 7 + call)
        big = torch.full((2 * n, 2 * n), float("nan"), dtype=torch.float64, device="cuda")
        big[::2, ::2] = A                    # element (i, j) at 4n*i + 2*j: rsa = 4n, csa = 2
        ldx = nrhs + 3
        X1 = torch.full((n, ldx), -7.0, dtype=torch.float64, device="cuda")
        X1[:, :nrhs] = B
        rc = L.ddla_dev_dtrsv_noalloc(C.c_void_p(stream.cuda_stream), uplo, trans, diag, n, nrhs,
                                      C.c_void_p(big.data_ptr()), 4 * n, 2, C.c_void_p(X1.data_ptr()), ldx)
        ddla._lib.check(rc, "dtrsv_noalloc")
        X2 = torch.full((n, ldx), -7.0, dtype=torch.float64, device="cuda")
        X2[:, :nrhs] = B
        rc = L.ddla_dev_dtrsm(h.h, LEFT, uplo, trans, diag, n, nrhs, 1.0, C.c_void_p(big.data_ptr()), 4 * n, 2,
                              C.c_void_p(X2.data_ptr()), ldx, 1)
        ddla._lib.check(rc, "dev_dtrsm")
        torch.cuda.synchronize()
        x1, x2 = X1.cpu().numpy(), X2.cpu().numpy()
        assert np.all(x1[:, nrhs:] == -7.0), "padding columns of X were written"
        assert np.max(np.abs(x1[:, :nrhs] - x2[:, :nrhs])) / np.abs(x2[:, :nrhs]).max() <= 1e-12
        a = A.cpu().numpy()
        T = np.tril(a) if uplo == LOWER else np.triu(a)
        if diag == UNIT:
            np.fill_diagonal(T, 1.0)
        op = T.T if trans == TRANS else T
        assert np.max(np.abs(op @ x1[:, :nrhs] - B.cpu().numpy())) <= 1e-12
    h.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(ddla):
    import torch
    L = ddla.lib()
    A = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = L.ddla_dev_dtrsv_noalloc(None, LOWER, NOTRANS, UNIT, 2049, 1, C.c_void_p(A.data_ptr()), 2049, 1,
                                  C.c_void_p(A.data_ptr()), 1)
    assert rc == -5 and b"exceeds" in L.ddla_last_error()
    rc = L.ddla_dev_dtrsv_noalloc(None, LOWER, NOTRANS, UNIT, 10, 17, C.c_void_p(A.data_ptr()), 10, 1,
                                  C.c_void_p(A.data_ptr()), 17)
    assert rc == -6
