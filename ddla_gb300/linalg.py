"""Host-side mirror of DDLA's BLAS provider and factorization classes over the
C ABI of libddla_gb300.

Names, argument order and error behaviour follow the reference so the parity
tests read like DDLA's own tests:

  BlasProvider.GeMM / GeMMT / SyRk / TrSM   DDLA/BLAS/3m.cs:10-315
  LU                                        DDLA/Factorizations/LU.cs:13-128
  Cholesky                                  DDLA/Factorizations/Cholesky.cs:10-88
  LDLT                                      DDLA/Factorizations/LDLT.cs:9-137
  QR                                        DDLA/Factorizations/QR.cs:14-534
  Tridiagonaling                            DDLA/Transformations/Tridiagonaling.cs:10-232
  Bidiagonaling.Bidiag (two-stage)          DDLA/Transformations/Bidiagonaling.cs:14-33, 334-582
  Bidiagonaling.Bidiag2                     DDLA/Transformations/Bidiagonaling.cs:35-143

Matrices are float64 numpy arrays; any 2-D view works (its element strides
are DDLA's RowStride / ColStride), and in-place operations write through the
view exactly as DDLA writes through a MatrixView.  Calls are synchronous.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import (LEFT, LOWER, NO_TRANSPOSE, NONUNIT, RIGHT, TRANSPOSE, UNIT, UPPER, LinalgError, Opts,
                   SolveReport, check, lib)

__all__ = ["BlasProvider", "LU", "Cholesky", "LDLT", "QR", "Tridiagonaling", "Bidiagonaling", "solve_mixed",
           "LinalgError"]


def _view(x, name):
    if not isinstance(x, np.ndarray) or x.dtype != np.float64:
        raise TypeError(f"{name} must be a float64 numpy array")
    if x.ndim == 1:
        x = x.reshape(-1, 1) if x.strides[0] else x[:, None]
    if x.ndim != 2:
        raise ValueError(f"{name} must be 2-D")
    return x


def _st(x):
    return x.strides[0] // 8, x.strides[1] // 8


def _p(x):
    return C.c_void_p(x.ctypes.data)


def _dims_after(x, trans):
    return (x.shape[1], x.shape[0]) if trans & TRANSPOSE else x.shape


class BlasProvider:
    """Level-3 calls with DDLA's checked-wrapper semantics (DDLA/BLAS/3m.cs)."""

    @staticmethod
    def GeMM(*args):
        """GeMM(aTrans, bTrans, alpha, A, B, beta, C) or GeMM(alpha, A, B, beta, C):
        C = beta*C + alpha*op(A)*op(B) (DDLA/BLAS/3m.cs:10-42)."""
        if len(args) == 5:
            args = (NO_TRANSPOSE, NO_TRANSPOSE) + tuple(args)
        ta, tb, alpha, A, B, beta, Cm = args
        A, B, Cm = _view(A, "A"), _view(B, "B"), _view(Cm, "C")
        m, n = Cm.shape
        if m == 0 or n == 0:
            return
        m2, k = _dims_after(A, ta)
        if k == 0:
            return
        if m2 != m:
            raise ValueError("Dimensions of matrix A must be match!")
        if _dims_after(B, tb) != (k, n):
            raise ValueError("Dimensions of matrix B must be match!")
        check(lib().ddla_dgemm(ta, tb, m, n, k, C.byref(C.c_double(alpha)), _p(A), *_st(A), _p(B), *_st(B),
                               C.byref(C.c_double(beta)), _p(Cm), *_st(Cm)), "GeMM")

    @staticmethod
    def GeMMT(*args):
        """GeMMT(cUplo, aTrans, bTrans, alpha, A, B, beta, C) or
        GeMMT(cUplo, alpha, A, B, beta, C) (DDLA/BLAS/3m.cs:44-81)."""
        if len(args) == 6:
            args = (args[0], NO_TRANSPOSE, NO_TRANSPOSE) + tuple(args[1:])
        uplo, ta, tb, alpha, A, B, beta, Cm = args
        A, B, Cm = _view(A, "A"), _view(B, "B"), _view(Cm, "C")
        m = Cm.shape[0]
        if Cm.shape[1] != m:
            raise ValueError("C must be square")
        if m == 0:
            return
        ma, k = _dims_after(A, ta)
        if k == 0:
            return
        if _dims_after(B, tb) != (k, m) or ma != m:
            raise ValueError("Dimensions of matrix A must be match!")
        check(lib().ddla_dgemmt(uplo, ta, tb, m, k, C.byref(C.c_double(alpha)), _p(A), *_st(A), _p(B), *_st(B),
                                C.byref(C.c_double(beta)), _p(Cm), *_st(Cm)), "GeMMT")

    @staticmethod
    def SyRk(*args):
        """SyRk(cUplo, aTrans, alpha, A, beta, C) or SyRk(cUplo, alpha, A, beta, C)
        (DDLA/BLAS/3m.cs:118-147)."""
        if len(args) == 5:
            args = (args[0], NO_TRANSPOSE) + tuple(args[1:])
        uplo, ta, alpha, A, beta, Cm = args
        A, Cm = _view(A, "A"), _view(Cm, "C")
        m = Cm.shape[0]
        if m == 0:
            return
        ma, k = _dims_after(A, ta)
        if k == 0:
            return
        if ma != m:
            raise ValueError("Dimensions of matrixs A must be match!")
        check(lib().ddla_dsyrk(uplo, ta, m, k, C.byref(C.c_double(alpha)), _p(A), *_st(A),
                               C.byref(C.c_double(beta)), _p(Cm), *_st(Cm)), "SyRk")

    @staticmethod
    def SyMM(*args):
        """SyMM(aSide, aUplo, bTrans, alpha, A, B, beta, C) or
        SyMM(aSide, aUplo, alpha, A, B, beta, C): C = beta C + alpha A op(B)
        (Left) or alpha op(B) A (Right), A symmetric in aUplo (DDLA/BLAS/3m.cs:83-116)."""
        if len(args) == 7:
            args = (args[0], args[1], NO_TRANSPOSE) + tuple(args[2:])
        side, uplo, tb, alpha, A, B, beta, Cm = args
        A, B, Cm = _view(A, "A"), _view(B, "B"), _view(Cm, "C")
        m, n = Cm.shape
        if m == 0 or n == 0:
            return
        if _dims_after(B, tb) != (m, n):
            raise ValueError("Dimensions of matrix B must be match!")
        if A.shape[0] != A.shape[1] or A.shape[0] != (m if side == LEFT else n):
            raise ValueError("Dimensions of matrixs must be match!")
        check(lib().ddla_dsymm(side, uplo, 0, tb, m, n, C.byref(C.c_double(alpha)), _p(A), *_st(A), _p(B),
                               *_st(B), C.byref(C.c_double(beta)), _p(Cm), *_st(Cm)), "SyMM")

    @staticmethod
    def SyR2k(*args):
        """SyR2k(cUplo, aTrans, bTrans, alpha, A, B, beta, C) or
        SyR2k(cUplo, alpha, A, B, beta, C): triangle of C = beta C +
        alpha (op(A) op(B)^T + op(B) op(A)^T) (DDLA/BLAS/3m.cs:149-183)."""
        if len(args) == 6:
            args = (args[0], NO_TRANSPOSE, NO_TRANSPOSE) + tuple(args[1:])
        uplo, ta, tb, alpha, A, B, beta, Cm = args
        A, B, Cm = _view(A, "A"), _view(B, "B"), _view(Cm, "C")
        m = Cm.shape[0]
        if Cm.shape[1] != m:
            raise ValueError("C must be square")
        if m == 0:
            return
        ma, k = _dims_after(A, ta)
        if k == 0:
            return
        if _dims_after(B, tb) != (m, k) or ma != m:
            raise ValueError("Dimensions of matrixs A and B must be match!")
        check(lib().ddla_dsyr2k(uplo, ta, tb, m, k, C.byref(C.c_double(alpha)), _p(A), *_st(A), _p(B), *_st(B),
                                C.byref(C.c_double(beta)), _p(Cm), *_st(Cm)), "SyR2k")

    @staticmethod
    def TrMM(*args):
        """TrMM(aSide, aUplo, aTrans, aDiag, alpha, A, B), TrMM(aSide, aUplo, aDiag,
        alpha, A, B) or TrMM(aSide, aUplo, alpha, A, B): B <- alpha op(A) B (Left)
        or alpha B op(A) (Right), A triangular (DDLA/BLAS/3m.cs:185-223)."""
        if len(args) == 5:
            args = (args[0], args[1], NO_TRANSPOSE, NONUNIT) + tuple(args[2:])
        elif len(args) == 6:
            args = (args[0], args[1], NO_TRANSPOSE) + tuple(args[2:])
        side, uplo, ta, diag, alpha, A, B = args
        A, B = _view(A, "A"), _view(B, "B")
        m, n = B.shape
        if m == 0 or n == 0:
            return
        if A.shape[0] != A.shape[1] or A.shape[0] != (m if side == LEFT else n):
            raise ValueError("Dimensions of matrixs A must be match!")
        check(lib().ddla_dtrmm(side, uplo, ta, diag, m, n, C.byref(C.c_double(alpha)), _p(A), *_st(A), _p(B),
                               *_st(B)), "TrMM")

    @staticmethod
    def TrMM3(*args):
        """TrMM3(aSide, aUplo, aTrans, aDiag, bTrans, alpha, A, B, beta, C),
        TrMM3(aSide, aUplo, aDiag, alpha, A, B, beta, C) or
        TrMM3(aSide, aUplo, alpha, A, B, beta, C): C = beta C + alpha op(A) op(B)
        (Left) or alpha op(B) op(A) (Right) (DDLA/BLAS/3m.cs:225-274)."""
        if len(args) == 7:
            args = (args[0], args[1], NO_TRANSPOSE, NONUNIT, NO_TRANSPOSE) + tuple(args[2:])
        elif len(args) == 8:
            args = (args[0], args[1], NO_TRANSPOSE, args[2], NO_TRANSPOSE) + tuple(args[3:])
        side, uplo, ta, diag, tb, alpha, A, B, beta, Cm = args
        A, B, Cm = _view(A, "A"), _view(B, "B"), _view(Cm, "C")
        m, n = Cm.shape
        if m == 0 or n == 0:
            return
        if _dims_after(B, tb) != (m, n):
            raise ValueError("Dimensions of matrix B must be match!")
        if A.shape[0] != A.shape[1] or A.shape[0] != (m if side == LEFT else n):
            raise ValueError("Dimensions of matrixs A must be match!")
        check(lib().ddla_dtrmm3(side, uplo, ta, diag, tb, m, n, C.byref(C.c_double(alpha)), _p(A), *_st(A), _p(B),
                                *_st(B), C.byref(C.c_double(beta)), _p(Cm), *_st(Cm)), "TrMM3")

    @staticmethod
    def TrSM(*args):
        """TrSM(aSide, aUplo, aTrans, aDiag, alpha, A, B) or TrSM(aSide, aUplo, alpha, A, B):
        B <- op(A)^-1 alpha B (Left) or alpha B op(A)^-1 (Right) (DDLA/BLAS/3m.cs:276-314)."""
        if len(args) == 5:
            args = (args[0], args[1], NO_TRANSPOSE, NONUNIT) + tuple(args[2:])
        side, uplo, ta, diag, alpha, A, B = args
        A, B = _view(A, "A"), _view(B, "B")
        m, n = B.shape
        if m == 0 or n == 0:
            return
        if A.shape[0] != A.shape[1] or A.shape[0] != (m if side == LEFT else n):
            raise ValueError("Dimensions of matrixs A must be match!")
        check(lib().ddla_dtrsm(side, uplo, ta, diag, m, n, C.byref(C.c_double(alpha)), _p(A), *_st(A), _p(B),
                               *_st(B)), "TrSM")


def _opts(nb=0, precision=0, max_iter=0, tol=0.0):
    o = Opts()
    o.nb, o.precision, o.max_iter, o.tol = nb, precision, max_iter, tol
    return o


class LU:
    """LU(A, inplace=False, usePiv=True) -- DDLA/Factorizations/LU.cs:13-128.
    Relative pivots: row i was swapped with row i + pivs[i]."""

    def __init__(self, A, inplace=False, usePiv=True):
        A = _view(A, "A")
        if A.shape[0] != A.shape[1]:
            raise ValueError("A must be square")
        self.n = A.shape[0]
        self.matrix = A if inplace else A.copy()
        self.pivs = np.zeros(self.n, dtype=np.int32) if usePiv else None
        self.computed = False
        self.deconstructed = False

    def _compute_once(self):
        if self.deconstructed:
            raise RuntimeError("Matrix has been deconstructed, cannot compute again.")
        if self.computed:
            return
        if self.pivs is None:
            LU.LUDecompose(self.matrix)
        else:
            LU.PLUDecompose(self.matrix, self.pivs)
        self.computed = True

    def Solve(self, b, trans=False, inplace=False):
        self._compute_once()
        vec = b.ndim == 1
        B = b if inplace else b.copy()
        B2 = _view(B, "b")
        if B2.shape[0] != self.n:
            raise ValueError("RHS vector size mismatch")
        if self.pivs is None:
            LU.LUSolve(self.matrix, B2, trans)
        else:
            LU.PLUSolve(self.matrix, self.pivs, B2, trans)
        return B if not vec else B2[:, 0]

    def Deconstruct(self):
        self._compute_once()
        n = self.n
        P = np.eye(n)
        if self.pivs is not None:
            LU.ApplyPiv(P, self.pivs)
        L = np.tril(self.matrix, -1) + np.eye(n)
        U = np.triu(self.matrix)
        self.deconstructed = True
        return P, L, U

    @staticmethod
    def PLUDecompose(A, pivs, nb=0):
        A = _view(A, "A")
        n = A.shape[0]
        if n != A.shape[1]:
            raise ValueError("Matrix must be square for LU factorization.")
        if len(pivs) != n:
            raise ValueError("The length of pivs must match the number of rows in the matrix.")
        if n == 0:
            return
        piv = np.zeros(n, dtype=np.int32)
        rc = lib().ddla_dgetrf(n, _p(A), *_st(A), C.c_void_p(piv.ctypes.data), C.byref(_opts(nb)))
        pivs[:] = piv
        check(rc, "PLUDecompose")

    @staticmethod
    def PLUSolve(A, pivs, B, trans=False):
        A, B = _view(A, "A"), _view(B, "B")
        n = A.shape[0]
        if B.shape[0] != n:
            raise ValueError("RHS matrix size mismatch")
        piv = np.ascontiguousarray(pivs, dtype=np.int32)
        check(lib().ddla_dgetrs(1 if trans else 0, n, B.shape[1], _p(A), *_st(A), C.c_void_p(piv.ctypes.data),
                                _p(B), *_st(B)), "PLUSolve")

    @staticmethod
    def LUDecompose(A, nb=0):
        A = _view(A, "A")
        if A.shape[0] != A.shape[1]:
            raise ValueError("Matrix must be square for LU factorization.")
        check(lib().ddla_dgetrf_nopiv(A.shape[0], _p(A), *_st(A), C.byref(_opts(nb))), "LUDecompose")

    @staticmethod
    def LUSolve(A, B, trans=False):
        A, B = _view(A, "A"), _view(B, "B")
        if B.shape[0] != A.shape[0]:
            raise ValueError("RHS matrix size mismatch")
        check(lib().ddla_dgetrs_nopiv(1 if trans else 0, A.shape[0], B.shape[1], _p(A), *_st(A), _p(B), *_st(B)),
              "LUSolve")

    @staticmethod
    def ApplyPiv(B, pivs, side=LEFT, forward=True):
        """Host-side row/column interchanges (LU.cs:237-249, 376-429)."""
        idx = range(len(pivs)) if forward else range(len(pivs) - 1, -1, -1)
        for i in idx:
            p = int(pivs[i])
            if p > 0:
                if side == LEFT:
                    B[[i, i + p]] = B[[i + p, i]]
                else:
                    B[:, [i, i + p]] = B[:, [i + p, i]]


class Cholesky:
    """Cholesky(A, uplo=Lower, inplace=False) -- DDLA/Factorizations/Cholesky.cs:10-88."""

    def __init__(self, A, uplo=LOWER, inplace=False):
        A = _view(A, "A")
        if A.shape[0] != A.shape[1]:
            raise ValueError("A must be square")
        self.uplo = uplo
        self.matrix = A if inplace else A.copy()
        self.computed = False

    def ComputeOnce(self):
        if self.computed:
            return
        self.computed = True
        Cholesky.CholDecompose(self.uplo, self.matrix)

    def Solve(self, b, inplace=False):
        self.ComputeOnce()
        vec = b.ndim == 1
        B = b if inplace else b.copy()
        B2 = _view(B, "b")
        Cholesky.CholeskySolve(self.uplo, self.matrix, B2)
        return B if not vec else B2[:, 0]

    @staticmethod
    def CholDecompose(uplo, A, nb=0):
        A = _view(A, "A")
        check(lib().ddla_dpotrf(uplo, A.shape[0], _p(A), *_st(A), C.byref(_opts(nb))), "Cholesky")

    @staticmethod
    def CholeskySolve(uplo, A, B):
        A, B = _view(A, "A"), _view(B, "B")
        if B.shape[0] != A.shape[0]:
            raise ValueError("Matrix dimensions do not match for Cholesky solve.")
        check(lib().ddla_dpotrs(uplo, A.shape[0], B.shape[1], _p(A), *_st(A), _p(B), *_st(B)), "CholeskySolve")


class LDLT:
    """LDLT(uplo, A, inplace=False) -- DDLA/Factorizations/LDLT.cs:9-137."""

    def __init__(self, uplo, A, inplace=False):
        A = _view(A, "A")
        if A.shape[0] != A.shape[1]:
            raise ValueError("A must be square")
        self.uplo = uplo
        self.matrix = A if inplace else A.copy()
        self.computed = False
        self.deconstructed = False

    def ComputeOnce(self):
        if self.deconstructed:
            raise RuntimeError("Matrix has been deconstructed, cannot compute again.")
        if self.computed:
            return
        self.computed = True
        LDLT.LDLTDecompose(self.uplo, self.matrix)

    def Solve(self, b, inplace=False):
        self.ComputeOnce()
        vec = b.ndim == 1
        B = b if inplace else b.copy()
        B2 = _view(B, "b")
        LDLT.LDLTSolve(self.uplo, self.matrix, B2)
        return B if not vec else B2[:, 0]

    def Deconstruct(self):
        self.ComputeOnce()
        D = np.diag(np.diag(self.matrix))
        n = self.matrix.shape[0]
        L = (np.tril(self.matrix, -1) if self.uplo == LOWER else np.triu(self.matrix, 1)) + np.eye(n)
        self.deconstructed = True
        return L, D

    @staticmethod
    def LDLTDecompose(uplo, A, nb=0):
        A = _view(A, "A")
        check(lib().ddla_dldlt(uplo, A.shape[0], _p(A), *_st(A), C.byref(_opts(nb))), "LDLT")

    @staticmethod
    def LDLTSolve(uplo, A, B):
        A, B = _view(A, "A"), _view(B, "B")
        if B.shape[0] != A.shape[0]:
            raise ValueError("Matrix dimensions do not match for Cholesky solve.")
        check(lib().ddla_dldlts(uplo, A.shape[0], B.shape[1], _p(A), *_st(A), _p(B), *_st(B)), "LDLTSolve")


class _InstanceOrStatic:
    """A name that is an instance method on instances and a static method on
    the class, like C#'s overloads QR.Solve(B) / QR.Solve(A, T, B, X)."""

    def __init__(self, inst, static):
        self.inst, self.static = inst, static

    def __get__(self, obj, objtype=None):
        if obj is None:
            return self.static
        return lambda *a, **k: self.inst(obj, *a, **k)


class QR:
    """QR(A, inplace=False) -- DDLA/Factorizations/QR.cs:14-122.  A is m x n
    (any m, n); Solve needs m >= n and returns the least-squares solution."""
    BlockSize = 256   # QR.cs:16

    def __init__(self, A, inplace=False):
        A = _view(A, "A")
        self.matrix = A if inplace else A.copy()
        self.aux = QR.CreateT(self.matrix)
        self.computed = False
        self.deconstructed = False

    def ComputeOnce(self):
        if self.deconstructed:
            raise RuntimeError("Matrix has been deconstructed, cannot compute again.")
        if self.computed:
            return
        self.computed = True
        QR.QRDecompose(self.matrix, self.aux)

    def _solve_inst(self, b, output=None):
        """QR.cs:45-77: the least-squares solution of A X = b."""
        self.ComputeOnce()
        vec = b.ndim == 1
        B = _view(b, "b")
        X = np.zeros((self.matrix.shape[1], B.shape[1])) if output is None else _view(output, "output")
        if X.shape != (self.matrix.shape[1], B.shape[1]):
            raise ValueError("Output matrix has incorrect dimensions.")
        QR._solve_static(self.matrix, self.aux, B, X)
        return X[:, 0] if vec else X

    def ApplyQ(self, b):
        """b <- Q b in place (QR.cs:79-93)."""
        B = _view(b, "b")
        QR.ApplyQlnfc(self.matrix, self.aux, B)
        return b

    def ApplyQT(self, b):
        """b <- Q^T b in place (QR.cs:95-109)."""
        B = _view(b, "b")
        QR.ApplyQlhfc(self.matrix, self.aux, B)
        return b

    def Deconstruct(self):
        """(Q m x m, R) as QR.cs:111-122."""
        self.ComputeOnce()
        m = self.matrix.shape[0]
        Q = np.zeros((m, m))
        QR.FormQ(self.matrix, self.aux, Q)
        R = np.triu(self.matrix)
        self.deconstructed = True
        return Q, R

    @staticmethod
    def CreateT(A):
        m, n = A.shape
        return np.zeros((min(QR.BlockSize, max(m, n)), n))

    @staticmethod
    def QRDecompose(A, T=None, precision=0, nb=0):
        A = _view(A, "A")
        if T is None:
            T = QR.CreateT(A)
        T = _view(T, "T")
        if T.shape[1] != A.shape[1]:
            raise ValueError("Matrix T and A must have the same number of columns.")
        check(lib().ddla_dgeqrf(A.shape[0], A.shape[1], _p(A), *_st(A), _p(T), T.shape[0], *_st(T),
                                C.byref(_opts(nb, precision))), "QRDecompose")
        return T

    @staticmethod
    def _solve_static(A, T, B, X):
        """QR.cs:151-168: X = argmin |A X - B| with the factors (A, T)."""
        A, T, B, X = _view(A, "A"), _view(T, "T"), _view(B, "B"), _view(X, "X")
        if A.shape[1] != T.shape[1]:
            raise ValueError("Matrix T and A must have the same number of columns.")
        if A.shape[0] != B.shape[0]:
            raise ValueError("Matrix A and B must have the same number of rows.")
        if A.shape[1] != X.shape[0]:
            raise ValueError("The number of columns in A must match the number of rows in X.")
        if X.shape[1] != B.shape[1]:
            raise ValueError("Matrix X and B must have the same number of columns.")
        m, n = A.shape
        check(lib().ddla_dgeqrs(m, n, B.shape[1], _p(A), *_st(A), _p(T), T.shape[0], *_st(T), _p(B), *_st(B),
                                _p(X), *_st(X)), "QR.Solve")

    Solve = _InstanceOrStatic(_solve_inst, _solve_static.__func__)

    @staticmethod
    def ApplyQlhfc(A, T, B):
        A, T, B = _view(A, "A"), _view(T, "T"), _view(B, "B")
        check(lib().ddla_dormqr(1, A.shape[0], A.shape[1], B.shape[1], _p(A), *_st(A), _p(T), T.shape[0], *_st(T),
                                _p(B), *_st(B)), "ApplyQlhfc")

    @staticmethod
    def ApplyQlnfc(A, T, B):
        A, T, B = _view(A, "A"), _view(T, "T"), _view(B, "B")
        check(lib().ddla_dormqr(0, A.shape[0], A.shape[1], B.shape[1], _p(A), *_st(A), _p(T), T.shape[0], *_st(T),
                                _p(B), *_st(B)), "ApplyQlnfc")

    @staticmethod
    def FormQ(A, T, Q):
        A, T, Q = _view(A, "A"), _view(T, "T"), _view(Q, "Q")
        if A.shape[1] != T.shape[1]:
            raise ValueError("Matrix T and A must have the same number of columns.")
        if Q.shape != (A.shape[0], A.shape[0]):
            raise ValueError("The dimension of Q must be equal to the number of rows in A.")
        check(lib().ddla_dorgqr(A.shape[0], A.shape[1], _p(A), *_st(A), _p(T), T.shape[0], *_st(T), _p(Q), *_st(Q)),
              "FormQ")


class Tridiagonaling:
    """Tridiagonaling.Tridiag -- DDLA/Transformations/Tridiagonaling.cs:10-232."""
    BlockSize = 64   # Tridiagonaling.cs:12

    @staticmethod
    def CreateT(A):
        n = A.shape[0]
        return np.zeros((min(Tridiagonaling.BlockSize, n), n))

    @staticmethod
    def Tridiag(A, T=None, d=None, e=None, precision=0):
        """Reduces the symmetric A (lower triangle read) in place: A <- Q with
        Q^T A Q = tridiag(d, e).  Returns (T, d, e)."""
        A = _view(A, "A")
        n = A.shape[0]
        if A.shape[1] != n:
            raise ValueError("A must be square")
        T = Tridiagonaling.CreateT(A) if T is None else _view(T, "T")
        d = np.zeros(n) if d is None else d
        e = np.zeros(max(n - 1, 0)) if e is None else e
        if T.shape[1] != n or d.shape != (n,) or e.shape != (max(n - 1, 0),):
            raise ValueError("T, d or e has the wrong shape")
        check(lib().ddla_dsytrd(n, _p(A), *_st(A), _p(T), T.shape[0], *_st(T), _p(d), _p(e) if n > 1 else None,
                                C.byref(_opts(0, precision))), "Tridiag")
        return T, d, e


class Bidiagonaling:
    """Bidiagonaling.Bidiag -- DDLA/Transformations/Bidiagonaling.cs:14-33
    (the two-stage reduction DDLA's SVD uses) and Bidiag2, :35-143 (the
    one-stage Householder reduction); both m >= n."""

    @staticmethod
    def Bidiag(A, precision=0):
        """Returns (U, V, d, e) with U^T A V = bidiag(d, e); A (m x n, m >= n)
        is left unchanged, as in DDLA (TwoStageBidiag works on a column-major
        clone, Bidiagonaling.cs:250-257)."""
        A = _view(A, "A")
        m, n = A.shape
        if m < n:
            raise ValueError("Only support m >= n")
        W = np.array(A, order="F")
        U, V = np.zeros((m, m), order="F"), np.zeros((n, n), order="F")
        d, e = np.zeros(n), np.zeros(max(n - 1, 0))
        check(lib().ddla_dbidiag_twostage(m, n, _p(W), *_st(W), _p(d), _p(e) if n > 1 else None, _p(U), *_st(U),
                                          _p(V), *_st(V), C.byref(_opts(0, precision))), "Bidiag")
        return U, V, d, e

    @staticmethod
    def Bidiag2(A, precision=0):
        """Returns (U, V, d, e) with U^T A V = bidiag(d, e); A (m x n, m >= n)
        is overwritten by the reflectors, as in DDLA."""
        A = _view(A, "A")
        m, n = A.shape
        if m < n:
            raise ValueError("Only support m >= n")
        U, V = np.zeros((m, m)), np.zeros((n, n))
        d, e = np.zeros(n), np.zeros(max(n - 1, 0))
        check(lib().ddla_dbidiag(m, n, _p(A), *_st(A), _p(d), _p(e) if n > 1 else None, _p(U), *_st(U), _p(V),
                                 *_st(V), C.byref(_opts(0, precision))), "Bidiag2")
        return U, V, d, e


def solve_mixed(A, B, spd=False, uplo=LOWER, precision=_lib.PREC_FP32, x_ref=None, tol=0.0, max_iter=0, nb=0,
                ldlt=False):
    """Mixed-precision solve with FP64 iterative refinement (no DDLA
    counterpart): LU (default), Cholesky (spd=True) or the unpivoted LDL^T of
    DDLA's LDLT (ldlt=True), any number of right-hand sides.  Returns
    (X, report dict with the growth monitor).  Raises on non-convergence."""
    A, B = _view(A, "A"), _view(B, "B")
    n, nrhs = B.shape
    X = np.zeros((n, nrhs))
    rep = SolveReport()
    xr = None if x_ref is None else np.ascontiguousarray(_view(x_ref, "x_ref"))
    xp = C.c_void_p(0) if xr is None else _p(xr)
    o = _opts(nb, precision, max_iter, tol)
    if ldlt:
        rc = lib().ddla_dsysv_mixed(uplo, n, nrhs, _p(A), *_st(A), _p(B), *_st(B), _p(X), *_st(X), xp, C.byref(o),
                                    C.byref(rep))
    elif spd:
        rc = lib().ddla_dposv_mixed(uplo, n, nrhs, _p(A), *_st(A), _p(B), *_st(B), _p(X), *_st(X), xp, C.byref(o),
                                    C.byref(rep))
    else:
        rc = lib().ddla_dgesv_mixed(n, nrhs, _p(A), *_st(A), _p(B), *_st(B), _p(X), *_st(X), xp, C.byref(o),
                                    C.byref(rep))
    check(rc, "solve_mixed")
    return X, rep.as_dict()
