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


def _declare_multi():
    L = _declare()
    if not getattr(L, "_einsum_declared", False):
        PP = C.POINTER(C.POINTER(_i64))
        L.ddla_einsum_path.argtypes = [C.c_char_p, C.c_int32, C.POINTER(C.c_int32), PP, C.c_char_p, C.c_int32]
        L.ddla_einsum_path.restype = C.c_int
        L.ddla_einsum.argtypes = [C.c_char_p, C.c_int32, C.POINTER(C.c_int32), PP, PP, C.POINTER(C.c_void_p),
                                  C.POINTER(_i64), C.c_double, C.c_double, C.c_int32, C.POINTER(_i64),
                                  C.POINTER(_i64), C.c_void_p, _i64, C.c_int32]
        L.ddla_einsum.restype = C.c_int
        L.ddla_dev_einsum.argtypes = [C.c_void_p, C.c_char_p, C.c_int32, C.POINTER(C.c_int32), PP, PP,
                                      C.POINTER(C.c_void_p), C.c_double, C.c_double, C.c_int32, C.POINTER(_i64),
                                      C.POINTER(_i64), C.c_void_p, C.c_int32]
        L.ddla_dev_einsum.restype = C.c_int
        L._einsum_declared = True
    return L


def _tables(shapes, strides=None):
    n = len(shapes)
    ranks = (C.c_int32 * n)(*[len(s) for s in shapes])
    keep = [_arr(list(s)) for s in shapes]
    lens = (C.POINTER(_i64) * n)(*[C.cast(k, C.POINTER(_i64)) for k in keep])
    sk, st = None, None
    if strides is not None:
        sk = [_arr(list(s)) for s in strides]
        st = (C.POINTER(_i64) * n)(*[C.cast(k, C.POINTER(_i64)) for k in sk])
    return ranks, lens, st, (keep, sk)


def _target_shape(expr, shapes):
    lhs, tgt = expr.replace(" ", "").split("->")
    dims = {}
    for name, shp in zip(lhs.split(","), shapes):
        for s, t in zip(name, shp):
            dims[s] = t
    return [dims[s] for s in tgt]


def einsum_path(expr, *operands):
    """DDLA's pairwise contraction order for `expr` (EinsumTree/EinsumState.cs:
    45-419) as a list of "ab,bc->ac" steps; operands are arrays or shapes."""
    shapes = [tuple(o.shape) if hasattr(o, "shape") else tuple(o) for o in operands]
    ranks, lens, _, keep = _tables(shapes)
    buf = C.create_string_buffer(4096)
    check(_declare_multi().ddla_einsum_path(expr.encode(), len(shapes), ranks, lens, buf, 4096), "einsum_path")
    s = buf.value.decode()
    return s.split(";") if s else []


def Einsum(expr, *operands, alpha=1.0, out=None, beta=0.0, precision=0):
    """MArray.Einsum (DDLA/Einsum/MArray.Contract.cs:409-427) on host arrays:
    out = beta*out + alpha*einsum(expr, operands).  Without `out` a new
    C-contiguous result is returned (DDLA's Einsum(expr, alpha, inputs));
    beta = 1 with `out` is DDLA's Einsum(result, expr, alpha, inputs)."""
    for i, x in enumerate(operands):
        _check_base(x, f"operand {i}")
    shapes = [x.shape for x in operands]
    if out is None:
        out = np.zeros(_target_shape(expr, shapes))
        beta = 0.0
    _check_base(out, "out")
    ranks, lens, strides, keep = _tables(shapes, [[s // 8 for s in x.strides] for x in operands])
    n = len(operands)
    ptrs = (C.c_void_p * n)(*[x.ctypes.data for x in operands])
    counts = (_i64 * n)(*[_span(x) for x in operands])
    lo, so = _arr(list(out.shape)), _arr([s // 8 for s in out.strides])
    check(_declare_multi().ddla_einsum(expr.encode(), n, ranks, lens, strides, ptrs, counts, float(alpha),
                                       float(beta), out.ndim, lo, so, C.c_void_p(out.ctypes.data), _span(out),
                                       precision), "Einsum")
    return out


def dev_einsum(handle, expr, operands, out, alpha=1.0, beta=0.0, precision=0):
    """The same on torch CUDA tensors (intermediates stay on the device)."""
    shapes = [tuple(x.shape) for x in operands]
    ranks, lens, strides, keep = _tables(shapes, [list(x.stride()) for x in operands])
    n = len(operands)
    ptrs = (C.c_void_p * n)(*[x.data_ptr() for x in operands])
    lo, so = _arr(list(out.shape)), _arr(list(out.stride()))
    check(_declare_multi().ddla_dev_einsum(handle.h, expr.encode(), n, ranks, lens, strides, ptrs, float(alpha),
                                           float(beta), out.dim(), lo, so, C.c_void_p(out.data_ptr()), precision),
          "dev_einsum")
    return out
