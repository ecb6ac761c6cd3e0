"""Batched small factorizations + solves (one persistent launch, CUDA graph).

Items are (A, b, kind) with kind 0 = LU with partial pivoting, 1 = LU without
pivoting, 2 = lower Cholesky.  torch provides the device buffers; the work is
done by libddla_gb300.so.
"""
import ctypes as C

import numpy as np

from ._lib import Opts, check, lib

KIND_PLU, KIND_LU, KIND_CHOL = 0, 1, 2


def _declare():
    L = lib()
    if not getattr(L, "_batched_declared", False):
        L.ddla_batched_plan_create.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int32,
                                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.POINTER(Opts), C.POINTER(C.c_void_p)]
        L.ddla_batched_plan_create.restype = C.c_int
        L.ddla_batched_plan_exec.argtypes = [C.c_void_p]
        L.ddla_batched_plan_exec.restype = C.c_int
        L.ddla_batched_plan_info.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32),
                                             C.POINTER(C.c_int64)]
        L.ddla_batched_plan_info.restype = C.c_int
        L.ddla_batched_plan_destroy.argtypes = [C.c_void_p]
        L.ddla_batched_plan_destroy.restype = C.c_int
        L._batched_declared = True
    return L


class BatchedSolver:
    """Packs the items into device buffers and builds the graph once; run()
    replays it (device-resident inputs)."""

    def __init__(self, handle, sizes, kinds, mixed, tol=0.0, max_iter=0, device="cuda"):
        import torch
        self.torch = torch
        self.h = handle
        self.sizes = np.asarray(sizes, dtype=np.int32)
        self.kinds = np.asarray(kinds, dtype=np.int32)
        self.mixed = bool(mixed)
        n2 = int((self.sizes.astype(np.int64) ** 2).sum())
        nv = int(self.sizes.sum())
        self.a = torch.zeros(max(n2, 1), dtype=torch.float64, device=device)
        self.a0 = torch.zeros_like(self.a)
        self.b = torch.zeros(max(nv, 1), dtype=torch.float64, device=device)
        self.x = torch.zeros_like(self.b)
        self.piv = torch.zeros(max(nv, 1), dtype=torch.int32, device=device)
        self.info = torch.zeros(max(len(sizes), 1), dtype=torch.int32, device=device)
        self.iters = torch.zeros_like(self.info)
        o = Opts()
        o.tol, o.max_iter = tol, max_iter
        self.plan = C.c_void_p()
        L = _declare()
        check(L.ddla_batched_plan_create(handle.h, len(sizes), self.sizes.ctypes.data, self.kinds.ctypes.data,
                                         1 if mixed else 0, self.a.data_ptr(), self.b.data_ptr(), self.x.data_ptr(),
                                         self.piv.data_ptr(), self.info.data_ptr(), self.iters.data_ptr(),
                                         C.byref(o), C.byref(self.plan)), "batched_plan_create")
        self.aoff = np.concatenate([[0], np.cumsum(self.sizes.astype(np.int64) ** 2)])
        self.voff = np.concatenate([[0], np.cumsum(self.sizes.astype(np.int64))])

    def load(self, mats, rhs):
        torch = self.torch
        A = np.concatenate([np.ascontiguousarray(m, dtype=np.float64).ravel() for m in mats])
        B = np.concatenate([np.asarray(v, dtype=np.float64).ravel() for v in rhs])
        self.a0.copy_(torch.from_numpy(A))
        self.b.copy_(torch.from_numpy(B))
        self.reset()

    def reset(self):
        """Restore the inputs (plain mode factors in place)."""
        if not self.mixed:
            self.a.copy_(self.a0)
        elif self.a.data_ptr() != self.a0.data_ptr():
            self.a.copy_(self.a0)

    def run(self):
        # inputs were written on torch's stream; the plan runs on the handle's
        self.torch.cuda.current_stream().synchronize()
        check(_declare().ddla_batched_plan_exec(self.plan), "batched_plan_exec")

    def info_tuple(self):
        fl, grid, sm = C.c_double(), C.c_int32(), C.c_int64()
        check(_declare().ddla_batched_plan_info(self.plan, C.byref(fl), C.byref(grid), C.byref(sm)), "plan_info")
        return fl.value, grid.value, sm.value

    def results(self):
        self.h.sync()
        a = self.a.cpu().numpy()
        x = self.x.cpu().numpy()
        piv = self.piv.cpu().numpy()
        out = []
        for i, n in enumerate(self.sizes):
            n = int(n)
            out.append((a[self.aoff[i]:self.aoff[i + 1]].reshape(n, n), x[self.voff[i]:self.voff[i + 1]],
                        piv[self.voff[i]:self.voff[i + 1]]))
        return out, self.info.cpu().numpy()[:len(self.sizes)], self.iters.cpu().numpy()[:len(self.sizes)]

    def close(self):
        if self.plan:
            _declare().ddla_batched_plan_destroy(self.plan)
            self.plan = C.c_void_p()
