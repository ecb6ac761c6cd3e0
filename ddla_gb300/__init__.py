"""GB300-native (sm_103a) implementation of DDLA's dense hot path.

The compute lives in libddla_gb300.so (hand-written CUDA kernels behind the C
ABI of include/ddla_gb300.h); this package is its host-side mirror of DDLA's
BlasProvider / LU / Cholesky / LDLT / QR / MArray.Contract interface.
"""
from ._lib import (DENSE, LEFT, LOWER, NO_TRANSPOSE, NONUNIT, PREC_BF16X3, PREC_FP32, PREC_FP64, PREC_OZAKI,
                   PREC_TF32X3, RIGHT, TRANSPOSE, UNIT, UPPER, DDLAError, LinalgError, kernel_launches, lib)
from .linalg import LDLT, LU, QR, BlasProvider, Bidiagonaling, Cholesky, Tridiagonaling, solve_mixed

__all__ = ["lib", "BlasProvider", "LU", "Cholesky", "LDLT", "QR", "Tridiagonaling", "Bidiagonaling", "solve_mixed", "LinalgError", "DDLAError",
           "kernel_launches", "NO_TRANSPOSE", "TRANSPOSE", "LOWER", "UPPER", "DENSE", "UNIT", "NONUNIT", "LEFT",
           "RIGHT", "PREC_FP64", "PREC_FP32", "PREC_TF32X3", "PREC_BF16X3", "PREC_OZAKI"]
