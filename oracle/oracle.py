"""ctypes front end of the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product library never does.  Each function takes numpy
float64 arrays (any strides: element strides are passed through exactly like
DDLA's MatrixView RowStride/ColStride) and mirrors the C entry points of
ddla_oracle.c, which restate DDLA's algorithms (see the citations there).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

TRANS_NO, TRANS_T = 0, 8
LOWER, UPPER, DENSE = 0xC0, 0x60, 0xE0
NONUNIT, UNIT = 0, 0x100
LEFT, RIGHT = 0, 1

_i64 = C.c_int64
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class ContractDesc(C.Structure):
    class Mode(C.Structure):
        _fields_ = [("len", _i64), ("sa", _i64), ("sb", _i64), ("sc", _i64)]

    _fields_ = [("nbatch", C.c_int), ("nm", C.c_int), ("nn", C.c_int), ("nk", C.c_int),
                ("swapped", C.c_int),
                ("batch", Mode * 48), ("m", Mode * 16), ("n", Mode * 16), ("k", Mode * 16)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        L = _lib
        L.orc_damax.restype = _i64
        L.orc_damax.argtypes = [_i64, _dp, _i64]
        for name in ("orc_dgetrf",):
            getattr(L, name).argtypes = [_i64, _dp, _i64, _i64, _ip]
        L.orc_dgetrf_nopiv.argtypes = [_i64, _dp, _i64, _i64]
        L.orc_dpotrf.argtypes = [C.c_int, _i64, _dp, _i64, _i64]
        L.orc_dldlt.argtypes = [C.c_int, _i64, _dp, _i64, _i64]
        L.orc_dgetrs.argtypes = [C.c_int, _i64, _i64, _dp, _i64, _i64, _ip, _dp, _i64, _i64]
        L.orc_dgetrs.restype = None
        L.orc_dgetrs_nopiv.argtypes = [C.c_int, _i64, _i64, _dp, _i64, _i64, _dp, _i64, _i64]
        L.orc_dgetrs_nopiv.restype = None
        L.orc_dpotrs.argtypes = [C.c_int, _i64, _i64, _dp, _i64, _i64, _dp, _i64, _i64]
        L.orc_dpotrs.restype = None
        L.orc_dldlts.argtypes = [C.c_int, _i64, _i64, _dp, _i64, _i64, _dp, _i64, _i64]
        L.orc_dgemm.argtypes = [C.c_int, C.c_int, _i64, _i64, _i64, C.c_double, _dp, _i64, _i64,
                                _dp, _i64, _i64, C.c_double, _dp, _i64, _i64]
        L.orc_dgemm.restype = None
        L.orc_dgemmt.argtypes = [C.c_int, C.c_int, C.c_int, _i64, _i64, C.c_double, _dp, _i64, _i64,
                                 _dp, _i64, _i64, C.c_double, _dp, _i64, _i64]
        L.orc_dgemmt.restype = None
        L.orc_dsyrk.argtypes = [C.c_int, C.c_int, _i64, _i64, C.c_double, _dp, _i64, _i64,
                                C.c_double, _dp, _i64, _i64]
        L.orc_dsyrk.restype = None
        L.orc_dtrsm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i64, _i64, C.c_double,
                                _dp, _i64, _i64, _dp, _i64, _i64]
        L.orc_dtrsm.restype = None
        L.orc_dsymm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i64, _i64, C.c_double, _dp, _i64, _i64,
                                _dp, _i64, _i64, C.c_double, _dp, _i64, _i64]
        L.orc_dsyr2k.argtypes = [C.c_int, C.c_int, C.c_int, _i64, _i64, C.c_double, _dp, _i64, _i64,
                                 _dp, _i64, _i64, C.c_double, _dp, _i64, _i64]
        L.orc_dtrmm3.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _i64, _i64, C.c_double,
                                 _dp, _i64, _i64, _dp, _i64, _i64, C.c_double, _dp, _i64, _i64]
        L.orc_dtrmm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i64, _i64, C.c_double,
                                _dp, _i64, _i64, _dp, _i64, _i64]
        L.orc_dgeqrf.argtypes = [_i64, _i64, _dp, _i64, _i64, _dp, _i64, _i64, _i64]
        L.orc_dormqr.argtypes = [C.c_int, _i64, _i64, _i64, _dp, _i64, _i64, _dp, _i64, _i64, _i64, _dp, _i64, _i64]
        L.orc_dgeqrs.argtypes = [_i64, _i64, _i64, _dp, _i64, _i64, _dp, _i64, _i64, _i64, _dp, _i64, _i64,
                                 _dp, _i64, _i64]
        L.orc_dorgqr.argtypes = [_i64, _i64, _dp, _i64, _i64, _dp, _i64, _i64, _i64, _dp, _i64, _i64]
        L.orc_dsytrd.argtypes = [_i64, _dp, _i64, _i64, _dp, _i64, _i64, _i64, _dp, _dp]
        L.orc_dbidiag.argtypes = [_i64, _i64, _dp, _i64, _i64, _dp, _i64, _dp, _i64, _dp, _dp, _dp, _i64, _i64,
                                  _dp, _i64, _i64]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_batched.argtypes = [_i64, _ip, _ip, _dp, _dp, _dp, _ip, _ip]
        L.orc_dbidiag2s.argtypes = [_i64, _i64, _dp, _i64, _i64, _dp, _i64, _i64, _dp, _i64, _i64, _dp, _dp]
        L.orc_batched.restype = None
        L.orc_contract_plan.argtypes = [C.c_char_p, C.c_int, C.POINTER(_i64), C.POINTER(_i64),
                                        C.c_int, C.POINTER(_i64), C.POINTER(_i64),
                                        C.c_int, C.POINTER(_i64), C.POINTER(_i64),
                                        C.POINTER(ContractDesc)]
        L.orc_contract_exec.argtypes = [C.POINTER(ContractDesc), C.c_double, _dp, _dp, _dp]
        L.orc_contract_exec.restype = None
        assert L.orc_contract_desc_size() == C.sizeof(ContractDesc)
    return _lib


def set_threads(n):
    lib().orc_set_threads(int(n))


def has_openmp():
    return bool(lib().orc_has_openmp())


def _ptr(x):
    assert x.dtype == np.float64
    return x.ctypes.data_as(_dp)


def _st(x):
    """Element strides (row, col) of a 2-D float64 array view."""
    return x.strides[0] // 8, x.strides[1] // 8


def damax(x):
    return int(lib().orc_damax(x.shape[0], _ptr(x), x.strides[0] // 8))


def dgemm(alpha, A, B, beta, Cm, ta=TRANS_NO, tb=TRANS_NO):
    m, n = Cm.shape
    k = A.shape[0] if ta == TRANS_T else A.shape[1]
    lib().orc_dgemm(ta, tb, m, n, k, alpha, _ptr(A), *_st(A), _ptr(B), *_st(B), beta, _ptr(Cm), *_st(Cm))


def dgemmt(uplo, alpha, A, B, beta, Cm, ta=TRANS_NO, tb=TRANS_NO):
    m = Cm.shape[0]
    k = A.shape[0] if ta == TRANS_T else A.shape[1]
    lib().orc_dgemmt(uplo, ta, tb, m, k, alpha, _ptr(A), *_st(A), _ptr(B), *_st(B), beta, _ptr(Cm), *_st(Cm))


def dsyrk(uplo, alpha, A, beta, Cm, ta=TRANS_NO):
    m = Cm.shape[0]
    k = A.shape[0] if ta == TRANS_T else A.shape[1]
    lib().orc_dsyrk(uplo, ta, m, k, alpha, _ptr(A), *_st(A), beta, _ptr(Cm), *_st(Cm))


def dsymm(side, uplo, alpha, A, B, beta, Cm, tb=TRANS_NO):
    m, n = Cm.shape
    lib().orc_dsymm(side, uplo, 0, tb, m, n, alpha, _ptr(A), *_st(A), _ptr(B), *_st(B), beta, _ptr(Cm), *_st(Cm))


def dsyr2k(uplo, alpha, A, B, beta, Cm, ta=TRANS_NO, tb=TRANS_NO):
    m = Cm.shape[0]
    k = A.shape[0] if ta == TRANS_T else A.shape[1]
    lib().orc_dsyr2k(uplo, ta, tb, m, k, alpha, _ptr(A), *_st(A), _ptr(B), *_st(B), beta, _ptr(Cm), *_st(Cm))


def dtrmm3(side, uplo, ta, diag, alpha, A, B, beta, Cm, tb=TRANS_NO):
    m, n = Cm.shape
    lib().orc_dtrmm3(side, uplo, ta, diag, tb, m, n, alpha, _ptr(A), *_st(A), _ptr(B), *_st(B), beta,
                     _ptr(Cm), *_st(Cm))


def dtrmm(side, uplo, ta, diag, alpha, A, B):
    m, n = B.shape
    lib().orc_dtrmm(side, uplo, ta, diag, m, n, alpha, _ptr(A), *_st(A), _ptr(B), *_st(B))


def qr_t_rows(m, n):
    """Rows of DDLA's T for an m x n QR (QR.CreateT, DDLA/Factorizations/QR.cs:124-128)."""
    return min(256, max(m, n))


def dgeqrf(A, T):
    """In-place QR of A; T (t_rows x n) receives the block factors."""
    m, n = A.shape
    rc = lib().orc_dgeqrf(m, n, _ptr(A), *_st(A), _ptr(T), T.shape[0], *_st(T))
    if rc:
        raise ValueError(f"orc_dgeqrf: argument {-rc}")


def dormqr(trans, A, T, B):
    m, n = A.shape
    lib().orc_dormqr(trans, m, n, B.shape[1], _ptr(A), *_st(A), _ptr(T), T.shape[0], *_st(T), _ptr(B), *_st(B))


def dgeqrs(A, T, B):
    m, n = A.shape
    X = np.zeros((n, B.shape[1]))
    lib().orc_dgeqrs(m, n, B.shape[1], _ptr(A), *_st(A), _ptr(T), T.shape[0], *_st(T), _ptr(B), *_st(B),
                     _ptr(X), *_st(X))
    return X


def dorgqr(A, T):
    m, n = A.shape
    Q = np.zeros((m, m))
    lib().orc_dorgqr(m, n, _ptr(A), *_st(A), _ptr(T), T.shape[0], *_st(T), _ptr(Q), *_st(Q))
    return Q


def trd_t_rows(n):
    """Rows of DDLA's T for a tridiagonal reduction (Tridiagonaling.CreateT, :15-19)."""
    return min(64, n)


def dsytrd(A, T):
    """Tridiag(A, T, d, e): A (lower triangle read) is overwritten by Q; returns (d, e)."""
    n = A.shape[0]
    d, e = np.zeros(n), np.zeros(max(n - 1, 1))
    lib().orc_dsytrd(n, _ptr(A), *_st(A), _ptr(T), T.shape[0], *_st(T), _ptr(d), _ptr(e))
    return d, e[:max(n - 1, 0)]


def bidiag(A):
    """Bidiagonaling.Bidiag2 (one stage, m >= n): returns (U, V, d, e, TU, TV)
    with U^T A V = bidiag(d, e); A is overwritten by the reflectors."""
    m, n = A.shape
    tur, tvr = min(128, n), max(min(128, n - 1), 1)
    TU, TV = np.zeros((tur, n)), np.zeros((tvr, n))
    d, e = np.zeros(n), np.zeros(max(n - 1, 1))
    U, V = np.zeros((m, m)), np.zeros((n, n))
    rc = lib().orc_dbidiag(m, n, _ptr(A), *_st(A), _ptr(TU), tur, _ptr(TV), tvr, _ptr(d), _ptr(e), _ptr(U), *_st(U),
                           _ptr(V), *_st(V))
    if rc:
        raise ValueError("orc_dbidiag: m < n")
    return U, V, d, e[:max(n - 1, 0)], TU, TV


def bidiag2s(A):
    """Bidiagonaling.Bidiag (two stages through TwoStageBidiag, m >= n):
    returns (U, V, d, e) with U^T A V = bidiag(d, e); A is overwritten."""
    m, n = A.shape
    U, V = np.zeros((m, m)), np.zeros((n, n))
    d, e = np.zeros(n), np.zeros(max(n - 1, 1))
    rc = lib().orc_dbidiag2s(m, n, _ptr(A), *_st(A), _ptr(U), *_st(U), _ptr(V), *_st(V), _ptr(d), _ptr(e))
    if rc:
        raise ValueError("orc_dbidiag2s: m < n")
    return U, V, d, e[:max(n - 1, 0)]


def dtrsm(side, uplo, ta, diag, alpha, A, B):
    m, n = B.shape
    lib().orc_dtrsm(side, uplo, ta, diag, m, n, alpha, _ptr(A), *_st(A), _ptr(B), *_st(B))


def dgetrf(A):
    """In-place PLU of A; returns (info, relative pivots int32[n])."""
    n = A.shape[0]
    piv = np.zeros(max(n, 1), dtype=np.int32)
    info = lib().orc_dgetrf(n, _ptr(A), *_st(A), piv.ctypes.data_as(_ip))
    return info, piv[:n]


def dgetrs(LU, piv, B, trans=0):
    piv = np.ascontiguousarray(piv, dtype=np.int32)
    lib().orc_dgetrs(trans, LU.shape[0], B.shape[1], _ptr(LU), *_st(LU), piv.ctypes.data_as(_ip), _ptr(B), *_st(B))


def dgetrf_nopiv(A):
    return lib().orc_dgetrf_nopiv(A.shape[0], _ptr(A), *_st(A))


def dgetrs_nopiv(LU, B, trans=0):
    lib().orc_dgetrs_nopiv(trans, LU.shape[0], B.shape[1], _ptr(LU), *_st(LU), _ptr(B), *_st(B))


def dpotrf(uplo, A):
    return lib().orc_dpotrf(uplo, A.shape[0], _ptr(A), *_st(A))


def dpotrs(uplo, Lf, B):
    lib().orc_dpotrs(uplo, Lf.shape[0], B.shape[1], _ptr(Lf), *_st(Lf), _ptr(B), *_st(B))


def dldlt(uplo, A):
    return lib().orc_dldlt(uplo, A.shape[0], _ptr(A), *_st(A))


def dldlts(uplo, F, B):
    return lib().orc_dldlts(uplo, F.shape[0], B.shape[1], _ptr(F), *_st(F), _ptr(B), *_st(B))


def _arr(v):
    return (_i64 * max(len(v), 1))(*v)


def contract_plan(expr, A, B, Cm):
    d = ContractDesc()
    sa = [s // 8 for s in A.strides]
    sb = [s // 8 for s in B.strides]
    sc = [s // 8 for s in Cm.strides]
    rc = lib().orc_contract_plan(expr.encode(), A.ndim, _arr(A.shape), _arr(sa), B.ndim, _arr(B.shape), _arr(sb),
                                 Cm.ndim, _arr(Cm.shape), _arr(sc), C.byref(d))
    if rc != 0:
        raise ValueError(f"contract plan failed ({rc}) for {expr!r}")
    return d


def contract(expr, alpha, A, B, Cm):
    """Cm += alpha * contraction(A, B) in place (MArray.Contract(result, ...))."""
    d = contract_plan(expr, A, B, Cm)
    lib().orc_contract_exec(C.byref(d), alpha, _ptr(A), _ptr(B), _ptr(Cm))
    return d


def plan_dict(d):
    def modes(arr, cnt):
        return [(arr[i].len, arr[i].sa, arr[i].sb, arr[i].sc) for i in range(cnt)]
    return {"batch": modes(d.batch, d.nbatch), "m": modes(d.m, d.nm), "n": modes(d.n, d.nn),
            "k": modes(d.k, d.nk), "swapped": d.swapped}


def einsum_path(expr, shapes):
    """DDLA's greedy pairwise order for a multi-operand einsum, restated from
    EinsumState (DDLA/Einsum/EinsumTree/EinsumState.cs:45-419): over all pairs
    (l < r) the smallest cost |result| - (|l| + |r|) wins, ties to the smaller
    l then r (OrderBy(Cost).ThenBy(Left + const), :362-368, stable); inputs
    count with size 0 (their size product starts at 0, :122-131); the result
    keeps the symbols of l and r that another tensor or the target uses, in
    first-appearance order, replaces l, and r is dropped (:162-260).  The last
    step writes the target (EinsumNodes.cs:82-93)."""
    lhs, target = expr.replace(" ", "").split("->")
    names = lhs.split(",")
    order, dims = [], {}
    for nm, shp in zip(names, shapes):
        for s, t in zip(nm, shp):
            if s not in dims:
                order.append(s)
                dims[s] = t
    sizes = [0.0] * len(names)
    steps = []
    while len(names) > 1:
        best = None
        for l in range(len(names) - 1):
            for r in range(l + 1, len(names)):
                others = set(target)
                for j, nm in enumerate(names):
                    if j not in (l, r):
                        others |= set(nm)
                out = "".join(s for s in order if (s in names[l] or s in names[r]) and s in others)
                rs = 1.0
                for s in out:
                    rs *= dims[s]
                cost = rs - (sizes[l] + sizes[r])
                if best is None or cost < best[0]:
                    best = (cost, l, r, out, rs)
        _, l, r, out, rs = best
        steps.append((names[l], names[r], out))
        names[l], sizes[l] = out, rs
        del names[r], sizes[r]
    if steps:
        steps[-1] = (steps[-1][0], steps[-1][1], target)
    return [f"{a},{b}->{c}" for a, b, c in steps]


def einsum(expr, operands):
    """Einsum with DDLA's path, every pairwise step through the oracle's
    MArray.Contract restatement (intermediates row-major over their symbols)."""
    lhs, target = expr.replace(" ", "").split("->")
    names = lhs.split(",")
    dims = {}
    for nm, x in zip(names, operands):
        for s, t in zip(nm, x.shape):
            dims[s] = t
    tensors = dict()
    cur = list(zip(names, operands))
    for step in einsum_path(expr, [x.shape for x in operands]):
        a, rest = step.split(",")
        b, out = rest.split("->")
        ia = next(i for i, (nm, _) in enumerate(cur) if nm == a)
        ib = next(i for i, (nm, _) in enumerate(cur) if nm == b and i != ia)
        A, B = cur[ia][1], cur[ib][1]
        R = np.zeros([dims[s] for s in out])
        contract(step, 1.0, np.ascontiguousarray(A), np.ascontiguousarray(B), R)
        cur[ia] = (out, R)
        del cur[ib]
    if len(operands) == 1:
        raise ValueError("oracle einsum: one operand (DDLA returns it unchanged)")
    return cur[0][1]


def batched(sizes, kinds, mats, rhs):
    """Factor and solve many small systems (orc_batched): returns per item
    (factors, x, relative pivots) and the info vector.  kinds: 0 PLU, 1 LU
    without pivoting, 2 lower Cholesky."""
    sizes = np.ascontiguousarray(sizes, dtype=np.int32)
    kinds = np.ascontiguousarray(kinds, dtype=np.int32)
    a = np.concatenate([np.ascontiguousarray(m, dtype=np.float64).ravel() for m in mats])
    b = np.concatenate([np.asarray(v, dtype=np.float64).ravel() for v in rhs])
    x = np.zeros_like(b)
    piv = np.zeros(b.shape[0], dtype=np.int32)
    info = np.zeros(len(sizes), dtype=np.int32)
    lib().orc_batched(len(sizes), sizes.ctypes.data_as(_ip), kinds.ctypes.data_as(_ip), _ptr(a), _ptr(b), _ptr(x),
                      piv.ctypes.data_as(_ip), info.ctypes.data_as(_ip))
    out, ao, vo = [], 0, 0
    for nn in sizes:
        nn = int(nn)
        out.append((a[ao:ao + nn * nn].reshape(nn, nn), x[vo:vo + nn], piv[vo:vo + nn]))
        ao += nn * nn
        vo += nn
    return out, info
