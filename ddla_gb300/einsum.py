"""MArray.Contract mirror: two-operand einsum on the GPU through the C ABI.

DDLA/Einsum/MArray.Contract.cs:
  Contract(result, expr, alpha, left, right)   result += alpha * left (x) right   (:48-125)
  Contract(beta, result, expr, alpha, l, r)    result = beta*result + ...          (:32-36)
  Contract(expr, alpha, left, right)           new result tensor                   (:131-250)
Tensors are float64 numpy arrays with any strides (DDLA's MArray carries
lengths and strides the same way, DDLA/Core/MArray/MArray.cs:70-95).
"""
import ctypes as C

import numpy as np

from ._lib import check, lib

_i64 = C.c_int64


class Mode(C.Structure):
    _fields_ = [("len", _i64), ("sa", _i64), ("sb", _i64), ("sc", _i64)]


class ContractDesc(C.Structure):
    _fields_ = [("nbatch", C.c_int32), ("nm", C.c_int32), ("nn", C.c_int32), ("nk", C.c_int32),
                ("swapped", C.c_int32), ("reserved", C.c_int32),
                ("batch", Mode * 48), ("m", Mode * 16), ("n", Mode * 16), ("k", Mode * 16)]

    def as_dict(self):
        def modes(arr, cnt):
            return [(arr[i].len, arr[i].sa, arr[i].sb, arr[i].sc) for i in range(cnt)]
        return {"batch": modes(self.batch, self.nbatch), "m": modes(self.m, self.nm), "n": modes(self.n, self.nn),
                "k": modes(self.k, self.nk), "swapped": self.swapped}


def _declare():
    L = lib()
    if not getattr(L, "_contract_declared", False):
        P = C.POINTER(_i64)
        L.ddla_contract_plan.argtypes = [C.c_char_p, C.c_int32, P, P, C.c_int32, P, P, C.c_int32, P, P,
                                         C.POINTER(ContractDesc)]
        L.ddla_contract_plan.restype = C.c_int
        L.ddla_contract.argtypes = [C.POINTER(ContractDesc), C.c_double, C.c_void_p, _i64, C.c_void_p, _i64,
                                    C.c_void_p, _i64, C.c_int32]
        L.ddla_contract.restype = C.c_int
        L.ddla_dev_contract.argtypes = [C.c_void_p, C.POINTER(ContractDesc), C.c_double, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_int32]
        L.ddla_dev_contract.restype = C.c_int
        L._contract_declared = True
    return L


def _arr(v):
    return (_i64 * max(len(v), 1))(*v)


def _lens_strides(x, elem=8):
    return list(x.shape), [s // elem for s in x.strides]


def plan(expr, A, B, Cshape_or_array, c_strides=None):
    """Index analysis only (host): returns the ContractDesc."""
    L = _declare()
    la, sa = _lens_strides(A)
    lb, sb = _lens_strides(B)
    if isinstance(Cshape_or_array, np.ndarray):
        lc, sc = _lens_strides(Cshape_or_array)
    else:
        lc, sc = list(Cshape_or_array), list(c_strides)
    d = ContractDesc()
    check(L.ddla_contract_plan(expr.encode(), len(la), _arr(la), _arr(sa), len(lb), _arr(lb), _arr(sb), len(lc),
                               _arr(lc), _arr(sc), C.byref(d)), "contract_plan")
    return d


def _span(x):
    """Elements spanned from x's first element (non-negative strides)."""
    if x.size == 0:
        return 0
    return int(sum((n - 1) * (s // 8) for n, s in zip(x.shape, x.strides))) + 1


def _check_base(x, name):
    if x.dtype != np.float64:
        raise TypeError(f"{name} must be float64")
    if any(s < 0 for s in x.strides):
        raise ValueError(f"{name}: negative strides are not supported")


def Contract(*args, precision=0):
    """Contract(result, expr, alpha, left, right) accumulates into result;
    Contract(expr, alpha, left, right) / Contract(expr, left, right) return a
    new C-contiguous result (DDLA MArray.Contract overloads)."""
    if isinstance(args[0], str):
        expr = args[0]
        alpha, left, right = (1.0, args[1], args[2]) if len(args) == 3 else args[1:4]
        lhs, out = expr.replace(" ", "").split("->")
        la, lb = lhs.split(",")
        dims = {}
        for s, t in zip(la, left.shape):
            dims[s] = t
        for s, t in zip(lb, right.shape):
            dims[s] = t
        result = np.zeros([dims[s] for s in out])
        Contract(result, expr, alpha, left, right, precision=precision)
        return result
    if isinstance(args[0], (int, float)) and len(args) == 6:
        beta, result, expr, alpha, left, right = args
        result *= beta
        return Contract(result, expr, alpha, left, right, precision=precision)
    result, expr, alpha, left, right = args
    for x, nm in ((left, "left"), (right, "right"), (result, "result")):
        _check_base(x, nm)
    d = plan(expr, left, right, result)
    check(_declare().ddla_contract(C.byref(d), float(alpha), C.c_void_p(left.ctypes.data), _span(left),
                                   C.c_void_p(right.ctypes.data), _span(right), C.c_void_p(result.ctypes.data),
                                   _span(result), precision), "Contract")
    return result
