"""Device-resident calls (ddla_dev_* entry points) on torch CUDA tensors.

torch is used only for device memory and streams; every computation is a call
into libddla_gb300.so.
"""
import ctypes as C

from . import _lib
from ._lib import Opts, SolveReport, check, lib


def _p(t):
    return C.c_void_p(t.data_ptr())


def _st(t):
    return t.stride(0), t.stride(1)


class Handle:
    """ddla_handle bound to a CUDA stream (torch.cuda.Stream or None)."""

    def __init__(self, stream=None):
        self.h = C.c_void_p()
        # torch reports the legacy default stream as 0, which the library reads
        # as "make a stream of your own": pass cudaStreamLegacy (1) instead
        s = None if stream is None else C.c_void_p(stream.cuda_stream or 1)
        check(lib().ddla_handle_create(C.byref(self.h), s), "handle_create")

    def close(self):
        if self.h:
            lib().ddla_handle_destroy(self.h)
            self.h = C.c_void_p()

    def sync(self):
        check(lib().ddla_handle_sync(self.h), "handle_sync")

    def gemm(self, alpha, A, B, beta, Cm, ta=0, tb=0, precision=None):
        """C = alpha op(A) op(B) + beta C; precision PREC_OZAKI selects the
        split BF16 tensor-core GEMM (FP64-level accuracy)."""
        m, n = Cm.shape
        k = A.shape[0] if ta else A.shape[1]
        if precision is None:
            check(lib().ddla_dev_dgemm(self.h, ta, tb, m, n, k, alpha, _p(A), *_st(A), _p(B), *_st(B), beta,
                                       _p(Cm), *_st(Cm)), "dev_dgemm")
        else:
            check(lib().ddla_dev_dgemm_ex(self.h, precision, ta, tb, m, n, k, alpha, _p(A), *_st(A), _p(B),
                                          *_st(B), beta, _p(Cm), *_st(Cm)), "dev_dgemm_ex")

    def gemmt(self, uplo, alpha, A, B, beta, Cm, ta=0, tb=0):
        m = Cm.shape[0]
        k = A.shape[0] if ta else A.shape[1]
        check(lib().ddla_dev_dgemmt(self.h, uplo, ta, tb, m, k, alpha, _p(A), *_st(A), _p(B), *_st(B), beta,
                                    _p(Cm), *_st(Cm)), "dev_dgemmt")

    def trsm(self, side, uplo, ta, diag, alpha, A, B):
        m, n = B.shape
        check(lib().ddla_dev_dtrsm(self.h, side, uplo, ta, diag, m, n, alpha, _p(A), *_st(A), _p(B), *_st(B)),
              "dev_dtrsm")

    def symm(self, side, uplo, alpha, A, B, beta, Cm, tb=0):
        m, n = Cm.shape
        check(lib().ddla_dev_dsymm(self.h, side, uplo, 0, tb, m, n, alpha, _p(A), *_st(A), _p(B), *_st(B), beta,
                                   _p(Cm), *_st(Cm)), "dev_dsymm")

    def syr2k(self, uplo, alpha, A, B, beta, Cm, ta=0, tb=0):
        m = Cm.shape[0]
        k = A.shape[0] if ta else A.shape[1]
        check(lib().ddla_dev_dsyr2k(self.h, uplo, ta, tb, m, k, alpha, _p(A), *_st(A), _p(B), *_st(B), beta,
                                    _p(Cm), *_st(Cm)), "dev_dsyr2k")

    def trmm(self, side, uplo, ta, diag, alpha, A, B):
        m, n = B.shape
        check(lib().ddla_dev_dtrmm(self.h, side, uplo, ta, diag, m, n, alpha, _p(A), *_st(A), _p(B), *_st(B)),
              "dev_dtrmm")

    def trmm3(self, side, uplo, ta, diag, alpha, A, B, beta, Cm, tb=0):
        m, n = Cm.shape
        check(lib().ddla_dev_dtrmm3(self.h, side, uplo, ta, diag, tb, m, n, alpha, _p(A), *_st(A), _p(B), *_st(B),
                                    beta, _p(Cm), *_st(Cm)), "dev_dtrmm3")

    def geqrf(self, A, T, precision=0, nb=0):
        m, n = A.shape
        o = Opts()
        o.precision, o.nb = precision, nb
        check(lib().ddla_dev_dgeqrf(self.h, m, n, _p(A), *_st(A), _p(T), T.shape[0], *_st(T), C.byref(o)),
              "dev_dgeqrf")

    def ormqr(self, trans, A, T, B):
        m, n = A.shape
        check(lib().ddla_dev_dormqr(self.h, 1 if trans else 0, m, n, B.shape[1], _p(A), *_st(A), _p(T), T.shape[0],
                                    *_st(T), _p(B), *_st(B)), "dev_dormqr")

    def geqrs(self, A, T, B, X):
        m, n = A.shape
        check(lib().ddla_dev_dgeqrs(self.h, m, n, B.shape[1], _p(A), *_st(A), _p(T), T.shape[0], *_st(T), _p(B),
                                    *_st(B), _p(X), *_st(X)), "dev_dgeqrs")

    def orgqr(self, A, T, Q):
        m, n = A.shape
        check(lib().ddla_dev_dorgqr(self.h, m, n, _p(A), *_st(A), _p(T), T.shape[0], *_st(T), _p(Q), *_st(Q)),
              "dev_dorgqr")

    def bidiag(self, A, d, e, U, V, precision=0):
        m, n = A.shape
        o = Opts()
        o.precision = precision
        check(lib().ddla_dev_dbidiag(self.h, m, n, _p(A), *_st(A), _p(d), _p(e) if n > 1 else None, _p(U), *_st(U),
                                     _p(V), *_st(V), C.byref(o)), "dev_dbidiag")

    def bidiag_twostage(self, A, d, e, U, V, precision=0):
        m, n = A.shape
        o = Opts()
        o.precision = precision
        check(lib().ddla_dev_dbidiag_twostage(self.h, m, n, _p(A), *_st(A), _p(d), _p(e) if n > 1 else None, _p(U),
                                              *_st(U), _p(V), *_st(V), C.byref(o)), "dev_dbidiag_twostage")

    def sytrd(self, A, T, d, e, precision=0):
        n = A.shape[0]
        o = Opts()
        o.precision = precision
        check(lib().ddla_dev_dsytrd(self.h, n, _p(A), *_st(A), _p(T), T.shape[0], *_st(T), _p(d),
                                    _p(e) if n > 1 else None, C.byref(o)), "dev_dsytrd")

    def getrf(self, A, piv, nb=0, precision=0):
        o = Opts()
        o.nb, o.precision = nb, precision
        return lib().ddla_dev_dgetrf(self.h, A.shape[0], _p(A), *_st(A), _p(piv), C.byref(o))

    def getrs(self, LU, piv, B, trans=0):
        check(lib().ddla_dev_dgetrs(self.h, trans, LU.shape[0], B.shape[1], _p(LU), *_st(LU), _p(piv), _p(B),
                                    *_st(B)), "dev_dgetrs")

    def potrf(self, uplo, A, nb=0, precision=0):
        o = Opts()
        o.nb, o.precision = nb, precision
        return lib().ddla_dev_dpotrf(self.h, uplo, A.shape[0], _p(A), *_st(A), C.byref(o))

    def potrs(self, uplo, A, B):
        check(lib().ddla_dev_dpotrs(self.h, uplo, A.shape[0], B.shape[1], _p(A), *_st(A), _p(B), *_st(B)),
              "dev_dpotrs")

    def gesv_mixed(self, A, B, X, x_ref=None, precision=_lib.PREC_FP32, tol=0.0, max_iter=0, nb=0, spd=False,
                   uplo=_lib.LOWER, piv_ref=None, piv_out=None, ldlt=False):
        """Mixed solve; for LU, piv_ref / piv_out (int32 device vectors of
        length n) compare the low-precision factor's pivots with a reference
        pivot vector and hand them out (ddla_dev_dgesv_mixed_piv)."""
        o = Opts()
        o.precision, o.tol, o.max_iter, o.nb = precision, tol, max_iter, nb
        rep = SolveReport()
        xr = C.c_void_p(0) if x_ref is None else _p(x_ref)
        n, nrhs = B.shape
        if ldlt:
            rc = lib().ddla_dev_dsysv_mixed(self.h, uplo, n, nrhs, _p(A), _p(B), _p(X), xr, C.byref(o), C.byref(rep))
        elif spd:
            rc = lib().ddla_dev_dposv_mixed(self.h, uplo, n, nrhs, _p(A), _p(B), _p(X), xr, C.byref(o), C.byref(rep))
        elif piv_ref is not None or piv_out is not None:
            rc = lib().ddla_dev_dgesv_mixed_piv(self.h, n, nrhs, _p(A), _p(B), _p(X), xr,
                                                C.c_void_p(0) if piv_ref is None else _p(piv_ref),
                                                C.c_void_p(0) if piv_out is None else _p(piv_out),
                                                C.byref(o), C.byref(rep))
        else:
            rc = lib().ddla_dev_dgesv_mixed(self.h, n, nrhs, _p(A), _p(B), _p(X), xr, C.byref(o), C.byref(rep))
        return rc, rep.as_dict()


def measure_peaks():
    f64, f32 = C.c_double(), C.c_double()
    check(lib().ddla_measure_peaks(C.byref(f64), C.byref(f32)), "measure_peaks")
    return f64.value, f32.value
