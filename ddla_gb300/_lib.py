"""ctypes binding of libddla_gb300.so (the C ABI in include/ddla_gb300.h).

The library is built in-tree (ddla_gb300/_build/) by ddla_gb300/build.py.
There is no fallback of any kind: if the shared library is missing or a call
fails, an exception is raised.
"""
import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libddla_gb300.so")

_lock = threading.Lock()
_lib = None

# flag values (DDLA/Misc/Flags/*.cs)
NO_TRANSPOSE, TRANSPOSE = 0, 8
LOWER, UPPER, DENSE = 0xC0, 0x60, 0xE0
NONUNIT, UNIT = 0x000, 0x100
LEFT, RIGHT = 0, 1

PREC_FP64, PREC_FP32, PREC_TF32X3, PREC_BF16X3, PREC_OZAKI = 0, 1, 2, 3, 4

ERR_CUDA, ERR_NOMEM, ERR_TIMEOUT, ERR_NOT_CONVERGED, ERR_UNSUPPORTED, ERR_NO_DEVICE = (
    -1001, -1002, -1003, -1004, -1005, -1006)


class LinalgError(ArithmeticError):
    """A factorization met a failing pivot (DDLA's LinalgException /
    ArgumentException from InvScal).  `index` is the 1-based pivot index."""

    def __init__(self, index, what="factorization"):
        super().__init__(f"{what}: failing pivot at index {index - 1} (0-based)")
        self.index = index


class DDLAError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ddla_gb300 error {code}: {msg}")
        self.code = code


class Opts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("nb", C.c_int32), ("max_iter", C.c_int32), ("reserved", C.c_int32),
                ("tol", C.c_double)]


class SolveReport(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("precision", C.c_int32),
                ("info", C.c_int32), ("backward_error", C.c_double), ("forward_error", C.c_double),
                ("factor_ms", C.c_double), ("refine_ms", C.c_double), ("pivots_agree", C.c_int32),
                ("pivots_first_diff", C.c_int32), ("growth", C.c_double), ("diag_ratio", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_i32, _i64, _d = C.c_int32, C.c_int64, C.c_double
_pd = C.c_void_p  # double* (host or device)
_pi = C.c_void_p  # int32*
_h = C.c_void_p

_SIGS = {
    "ddla_last_error": (C.c_char_p, []),
    "ddla_version": (C.c_char_p, []),
    "ddla_kernel_launches": (_i64, []),
    "ddla_handle_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p]),
    "ddla_handle_destroy": (C.c_int, [_h]),
    "ddla_handle_sync": (C.c_int, [_h]),
    "ddla_measure_peaks": (C.c_int, [C.POINTER(_d), C.POINTER(_d)]),
    "ddla_dev_sgemm_tc": (C.c_int, [_h, _i32, _i64, _i64, _i64, C.c_float, _pd, _i64, _i64, _pd, _i64, _i64,
                                    C.c_float, _pd, _i64, _i64]),
    "ddla_dev_dtrsv_noalloc": (C.c_int, [C.c_void_p, _i32, _i32, _i32, _i64, _i64, _pd, _i64, _i64, _pd, _i64]),
    "ddla_tune_set": (C.c_int, [C.c_char_p, _i64]),
    "ddla_tune_get": (_i64, [C.c_char_p, _i64]),
    "ddla_timing_enable": (C.c_int, [C.c_int]),
    "ddla_timing_read": (C.c_int, [C.c_int, C.POINTER(_d), C.POINTER(_i64), C.POINTER(_d), C.POINTER(_d)]),
    "ddla_dgemm": (C.c_int, [_i32, _i32, _i64, _i64, _i64, C.POINTER(_d), _pd, _i64, _i64, _pd, _i64, _i64,
                             C.POINTER(_d), _pd, _i64, _i64]),
    "ddla_dgemmt": (C.c_int, [_i32, _i32, _i32, _i64, _i64, C.POINTER(_d), _pd, _i64, _i64, _pd, _i64, _i64,
                              C.POINTER(_d), _pd, _i64, _i64]),
    "ddla_dsyrk": (C.c_int, [_i32, _i32, _i64, _i64, C.POINTER(_d), _pd, _i64, _i64, C.POINTER(_d), _pd, _i64,
                             _i64]),
    "ddla_dtrsm": (C.c_int, [_i32, _i32, _i32, _i32, _i64, _i64, C.POINTER(_d), _pd, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dsymm": (C.c_int, [_i32, _i32, _i32, _i32, _i64, _i64, C.POINTER(_d), _pd, _i64, _i64, _pd, _i64, _i64,
                             C.POINTER(_d), _pd, _i64, _i64]),
    "ddla_dsyr2k": (C.c_int, [_i32, _i32, _i32, _i64, _i64, C.POINTER(_d), _pd, _i64, _i64, _pd, _i64, _i64,
                              C.POINTER(_d), _pd, _i64, _i64]),
    "ddla_dtrmm": (C.c_int, [_i32, _i32, _i32, _i32, _i64, _i64, C.POINTER(_d), _pd, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dtrmm3": (C.c_int, [_i32, _i32, _i32, _i32, _i32, _i64, _i64, C.POINTER(_d), _pd, _i64, _i64, _pd, _i64,
                              _i64, C.POINTER(_d), _pd, _i64, _i64]),
    "ddla_dgeqrf": (C.c_int, [_i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _i64, C.POINTER(Opts)]),
    "ddla_dormqr": (C.c_int, [_i32, _i64, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dgeqrs": (C.c_int, [_i64, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _i64, _pd, _i64, _i64, _pd, _i64,
                              _i64]),
    "ddla_dorgqr": (C.c_int, [_i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dev_dgeqrf": (C.c_int, [_h, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _i64, C.POINTER(Opts)]),
    "ddla_dev_dormqr": (C.c_int, [_h, _i32, _i64, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _i64, _pd, _i64,
                                  _i64]),
    "ddla_dev_dgeqrs": (C.c_int, [_h, _i64, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _i64, _pd, _i64, _i64,
                                  _pd, _i64, _i64]),
    "ddla_dev_dorgqr": (C.c_int, [_h, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dsytrd": (C.c_int, [_i64, _pd, _i64, _i64, _pd, _i64, _i64, _i64, _pd, _pd, C.POINTER(Opts)]),
    "ddla_dev_dsytrd": (C.c_int, [_h, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _i64, _pd, _pd, C.POINTER(Opts)]),
    "ddla_dbidiag": (C.c_int, [_i64, _i64, _pd, _i64, _i64, _pd, _pd, _pd, _i64, _i64, _pd, _i64, _i64,
                               C.POINTER(Opts)]),
    "ddla_dev_dbidiag": (C.c_int, [_h, _i64, _i64, _pd, _i64, _i64, _pd, _pd, _pd, _i64, _i64, _pd, _i64, _i64,
                                   C.POINTER(Opts)]),
    "ddla_dbidiag_twostage": (C.c_int, [_i64, _i64, _pd, _i64, _i64, _pd, _pd, _pd, _i64, _i64, _pd, _i64, _i64,
                                        C.POINTER(Opts)]),
    "ddla_dev_dbidiag_twostage": (C.c_int, [_h, _i64, _i64, _pd, _i64, _i64, _pd, _pd, _pd, _i64, _i64, _pd, _i64,
                                            _i64, C.POINTER(Opts)]),
    "ddla_dgetrf": (C.c_int, [_i64, _pd, _i64, _i64, _pi, C.POINTER(Opts)]),
    "ddla_dgetrs": (C.c_int, [_i32, _i64, _i64, _pd, _i64, _i64, _pi, _pd, _i64, _i64]),
    "ddla_dgetrf_nopiv": (C.c_int, [_i64, _pd, _i64, _i64, C.POINTER(Opts)]),
    "ddla_dgetrs_nopiv": (C.c_int, [_i32, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dpotrf": (C.c_int, [_i32, _i64, _pd, _i64, _i64, C.POINTER(Opts)]),
    "ddla_dpotrs": (C.c_int, [_i32, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dldlt": (C.c_int, [_i32, _i64, _pd, _i64, _i64, C.POINTER(Opts)]),
    "ddla_dldlts": (C.c_int, [_i32, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dgesv_mixed": (C.c_int, [_i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _pd,
                                   C.POINTER(Opts), C.POINTER(SolveReport)]),
    "ddla_dposv_mixed": (C.c_int, [_i32, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _pd,
                                   C.POINTER(Opts), C.POINTER(SolveReport)]),
    "ddla_dev_dgemm": (C.c_int, [_h, _i32, _i32, _i64, _i64, _i64, _d, _pd, _i64, _i64, _pd, _i64, _i64, _d, _pd,
                                 _i64, _i64]),
    "ddla_dev_dgemm_ex": (C.c_int, [_h, _i32, _i32, _i32, _i64, _i64, _i64, _d, _pd, _i64, _i64, _pd, _i64, _i64,
                                    _d, _pd, _i64, _i64]),
    "ddla_dev_dgemmt": (C.c_int, [_h, _i32, _i32, _i32, _i64, _i64, _d, _pd, _i64, _i64, _pd, _i64, _i64, _d, _pd,
                                  _i64, _i64]),
    "ddla_dev_dtrsm": (C.c_int, [_h, _i32, _i32, _i32, _i32, _i64, _i64, _d, _pd, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dev_dsymm": (C.c_int, [_h, _i32, _i32, _i32, _i32, _i64, _i64, _d, _pd, _i64, _i64, _pd, _i64, _i64, _d,
                                 _pd, _i64, _i64]),
    "ddla_dev_dsyr2k": (C.c_int, [_h, _i32, _i32, _i32, _i64, _i64, _d, _pd, _i64, _i64, _pd, _i64, _i64, _d, _pd,
                                  _i64, _i64]),
    "ddla_dev_dtrmm": (C.c_int, [_h, _i32, _i32, _i32, _i32, _i64, _i64, _d, _pd, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dev_dtrmm3": (C.c_int, [_h, _i32, _i32, _i32, _i32, _i32, _i64, _i64, _d, _pd, _i64, _i64, _pd, _i64,
                                  _i64, _d, _pd, _i64, _i64]),
    "ddla_dev_dgetrf": (C.c_int, [_h, _i64, _pd, _i64, _i64, _pi, C.POINTER(Opts)]),
    "ddla_dev_dgetrs": (C.c_int, [_h, _i32, _i64, _i64, _pd, _i64, _i64, _pi, _pd, _i64, _i64]),
    "ddla_dev_dpotrf": (C.c_int, [_h, _i32, _i64, _pd, _i64, _i64, C.POINTER(Opts)]),
    "ddla_dev_dpotrs": (C.c_int, [_h, _i32, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dev_dldlt": (C.c_int, [_h, _i32, _i64, _pd, _i64, _i64, C.POINTER(Opts)]),
    "ddla_dev_dldlts": (C.c_int, [_h, _i32, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64]),
    "ddla_dev_dgesv_mixed": (C.c_int, [_h, _i64, _i64, _pd, _pd, _pd, _pd, C.POINTER(Opts),
                                       C.POINTER(SolveReport)]),
    "ddla_dev_dposv_mixed": (C.c_int, [_h, _i32, _i64, _i64, _pd, _pd, _pd, _pd, C.POINTER(Opts),
                                       C.POINTER(SolveReport)]),
    "ddla_dev_dgesv_mixed_piv": (C.c_int, [_h, _i64, _i64, _pd, _pd, _pd, _pd, _pi, _pi, C.POINTER(Opts),
                                           C.POINTER(SolveReport)]),
    "ddla_dev_dsysv_mixed": (C.c_int, [_h, _i32, _i64, _i64, _pd, _pd, _pd, _pd, C.POINTER(Opts),
                                       C.POINTER(SolveReport)]),
    "ddla_dsysv_mixed": (C.c_int, [_i32, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _pd, _i64, _i64, _pd,
                                   C.POINTER(Opts), C.POINTER(SolveReport)]),
}


def lib():
    """Load (once) and return the CDLL with every signature declared."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run ddla_gb300/build.py (the CUDA library is required; "
                              "there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_names():
    """C entry points bound by this package (here and in einsum.py / batched.py)."""
    import re
    names = set(_SIGS)
    for mod in ("einsum.py", "batched.py"):
        src = open(os.path.join(HERE, mod)).read()
        names |= set(re.findall(r"L\.(ddla_[a-z0-9_]+)\.argtypes", src))
    return sorted(names)


def last_error():
    return lib().ddla_last_error().decode(errors="replace")


def check(rc, what="call"):
    """Map a status code to an exception (0 passes)."""
    if rc == 0:
        return 0
    if rc > 0:
        raise LinalgError(rc, what)
    if rc > -1000:
        raise ValueError(f"{what}: invalid argument {-rc}: {last_error()}")
    raise DDLAError(rc, f"{what}: {last_error()}")


def kernel_launches():
    return int(lib().ddla_kernel_launches())
