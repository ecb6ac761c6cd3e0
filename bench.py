"""Benchmark: mixed-precision LU solve with FP64 iterative refinement on one GB300.

Workload (the configuration the headline metric is quoted on): A n x n with
i.i.d. N(0,1) entries, n = 8192, one right-hand side b ~ N(0,1); LU with
partial pivoting in FP32 storage with trailing updates in the selected
precision, then FP64 refinement on the GPU until the relative backward error
max ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= 1e-14.

A step = one complete solve (FP64 -> FP32 conversion, factorization, initial
solve, refinement loop) from the FP64 A and b resident in HBM.  The default
precision is FP32 storage with 3xTF32 tensor-core trailing updates; the
refinement for one right-hand side is flexible GMRES in FP64 preconditioned
by the FP32 factors.  The credited
work is the algorithmic LU+solve count 2/3 n^3 + 2 n^2 flops (refinement flops
are not credited).  A step only counts if it reaches the tolerance.

  value   device throughput, inputs resident, CUDA events on the solve stream
  e2e     the same through the host C ABI (ddla_dgesv_mixed) with pinned host
          buffers: host->device copy of A and b, solve, device->host copy of x
  roofline  the dominant kernel class, timed per launch with CUDA events
  cpu_baseline  the oracle (C restatement of DDLA's managed LU + solve) on the
          host cores, bounded sample

--impl reference times that CPU restatement as the reference arm.
--gpus N (torchrun, one rank per GPU) runs N independent replicas: the solve
does not shard across devices.

--workload selects one of the other configurations instead (device-resident
timing lines used for the per-kernel measurements and profiles; the default
is the headline LU solve):
  gemm      C = A B + 0.5 C, 1024^3, U[-1,1]      (--precision fp64 | ozaki)
  chol      SPD G G^T/n + I, n = 16384, 16 RHS    (--precision fp32 | fp64 | ...)
  batched   20,000 LU / Cholesky solves, n ~ U{8..256}  (--precision fp32 | fp64)
  einsum-a  'bik,bkj->bij', b = 512, 256^3, U[-1,1]  (--precision fp64 | ozaki)
  einsum-b  'abcd,cdef->abef', all lengths 64        (--precision fp64 | ozaki)
  bidiag2s  two-stage bidiagonal reduction + U, V, 4096^2 U[-1,1]  (--precision fp64 | ozaki)
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 8192
SEED = 0xDD1A0002
TOL = 1e-14
# DRAM bytes (read + write) of one k_panel_lu launch from the ncu capture in
# profiles/k_panel_lu_fp32_n8192.md (panel of 6912 x 64 FP32)
PANEL_TRAFFIC = 1.81e6
METRIC = "Solve GFLOP/s at FP64-level residual: mixed+refined vs plain FP64, 1 GB300"
UNIT = "GFLOP/s"


def lu_flops(n, nrhs=1):
    return 2.0 / 3.0 * n ** 3 + 2.0 * n ** 2 * nrhs


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def apply_tune(args):
    """--tune KEY=VALUE options -> the library's tuning table."""
    from ddla_gb300 import autotune
    for kv in args.tune:
        k, v = kv.split("=", 1)
        autotune.tune_set(k, int(v))


def max_over_ranks(ms, world, device="cuda"):
    """Step time of the job: the slowest rank's (all ranks get it)."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(flops_per_rank, world, ms):
    """Whole-job GFLOP/s of `world` independent replicas (weak scaling)."""
    return flops_per_rank * world / (ms * 1e-3) / 1e9


class ClockSampler:
    """nvidia-smi sampler running while the timed region runs."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "samples": len(sm),
                "reasons": sorted(reasons)}


def headline_inputs(n, seed):
    """A (n x n) and b (n x 1), i.i.d. N(0,1) from a seeded host generator, so
    that the GPU arm, the oracle checks and the reference arm all solve the
    same system."""
    import numpy as np
    r = np.random.default_rng(seed)
    A = r.standard_normal((n, n))
    b = r.standard_normal((n, 1))
    return A, b


def headline_config(n, world):
    """The workload both arms report (the problem, not the method)."""
    return {"workload": f"LU (partial pivoting) + solve, n={n}, 1 RHS, A and b i.i.d. N(0,1) from a fixed seed, "
                        f"to relative backward error <= {TOL:g}",
            "n": n, "nrhs": 1, "tol": TOL, "parallelism": f"replicas{world}", "l2": "inputs larger than L2"}


def oracle_solve(A, b, threads):
    """Oracle LU + solve (DDLA's managed algorithm restated in C): factors,
    relative pivots, x and the wall time."""
    from oracle import oracle
    oracle.set_threads(threads)
    F = A.copy()
    x = b.copy()
    t = time.perf_counter()
    info, piv = oracle.dgetrf(F)
    oracle.dgetrs(F, piv, x)
    dt = time.perf_counter() - t
    if info != 0:
        raise RuntimeError(f"oracle dgetrf failed at pivot {info}")
    return F, piv, x, dt


def reference_arm(args):
    """The reference's CPU path on this machine's host cores: DDLA's managed LU +
    solve (the oracle's C restatement), all host threads, on the headline
    workload itself (same n, same seeded A and b)."""
    rank, world, _ = dist_env()
    if world > 1 and rank != 0:
        return
    cores = os.cpu_count() or 1
    n = args.n
    A, b = headline_inputs(n, SEED)
    times = []
    for i in range(args.warmup + args.steps):
        if i < args.warmup:
            # warm-up: a small solve brings up the thread pool and the pages of
            # the library; the full-size solves are all timed
            oracle_solve(A[:512, :512].copy(), b[:512].copy(), cores)
            continue
        _, _, _, dt = oracle_solve(A, b, cores)
        times.append(dt)
    ms = statistics.median(times) * 1e3
    value = lu_flops(n) / (ms * 1e-3) / 1e9
    out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic N(0,1), seeded",
           "config": headline_config(n, 1),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": f"oracle dgetrf+dgetrs (C restatement of DDLA's managed blocked LU, nb = 128) "
                                      f"on the full n={n} system, {cores} OpenMP threads, one solve per timed step "
                                      f"(median of {args.steps}); warm-up steps are n=512 solves"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


class L2Flush:
    """Writes a buffer larger than L2 (129 MB) between timed steps of
    workloads whose inputs fit in L2."""

    def __init__(self, torch, stream):
        self.buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MB
        self.stream = stream

    def __call__(self):
        self.buf.fill_(1.0)


def secondary(args):
    """Device-resident lines for the other configurations (same JSON keys)."""
    import numpy as np
    import torch
    import ddla_gb300 as D
    from ddla_gb300 import batched as bt
    from ddla_gb300 import build as bld
    from ddla_gb300 import device as dv
    from ddla_gb300 import einsum as es
    bld.build()
    L = D.lib()
    apply_tune(args)
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    h = dv.Handle(stream)
    g = torch.Generator(device="cuda").manual_seed(SEED + 10)
    wl = args.workload
    pname = args.precision if args.precision != "auto" else ("fp32" if wl in ("chol", "batched") else "fp64")
    prec = {"fp32": D.PREC_FP32, "tf32x3": D.PREC_TF32X3, "bf16x3": D.PREC_BF16X3, "fp64": D.PREC_FP64,
            "ozaki": D.PREC_OZAKI}[pname]
    flush = None
    check_err = None
    bytes_alg = 0.0
    last_rep = {}

    def U(*shape):
        return torch.rand(*shape, dtype=torch.float64, device="cuda", generator=g) * 2 - 1

    if wl == "gemm":
        n = 1024
        A, B, C0 = U(n, n), U(n, n), U(n, n)
        Cm = C0.clone()
        flops = 2.0 * n ** 3
        bytes_alg = 8.0 * 4 * n * n
        flush = L2Flush(torch, stream)
        desc = f"GEMM C = A B + 0.5 C, {n}^3 FP64 row-major U[-1,1], {pname}"

        def step():
            h.gemm(1.0, A, B, 0.5, Cm, precision=prec)

        def check_err():
            ref = A @ B + 0.5 * C0            # accuracy check only, outside the timed region
            Cm.copy_(C0)
            step()
            return float(((Cm - ref).abs() / (A.abs() @ B.abs() + 0.5 * C0.abs())).max())
    elif wl in ("symm", "trmm", "syr2k"):
        n = args.n if args.n != N_DEFAULT else 4096
        A, B, C0 = U(n, n), U(n, n), U(n, n)
        Cm = C0.clone()
        flush = L2Flush(torch, stream)
        if wl == "symm":
            flops = 2.0 * n ** 3
            desc = f"SYMM C = A_sym B + 0.5 C (left, lower), {n}^3 FP64 U[-1,1]"

            def step():
                h.symm(D.LEFT, D.LOWER, 1.0, A, B, 0.5, Cm)

            def ref_fn():
                S = torch.tril(A) + torch.tril(A, -1).T
                return S @ B + 0.5 * C0, S.abs() @ B.abs() + 0.5 * C0.abs()
        elif wl == "trmm":
            flops = 1.0 * n ** 3
            desc = f"TRMM B = U B in place (left, upper, non-unit), {n}^3 FP64 U[-1,1]"

            def step():
                h.trmm(D.LEFT, D.UPPER, 0, 0, 1.0, A, Cm)

            def ref_fn():
                Tu = torch.triu(A)
                return Tu @ C0, Tu.abs() @ C0.abs()
        else:
            flops = 2.0 * n ** 3
            desc = f"SYR2K lower(C) = A B^T + B A^T + 0.5 C, m = k = {n}, FP64 U[-1,1]"

            def step():
                h.syr2k(D.LOWER, 1.0, A, B, 0.5, Cm)

            def ref_fn():
                return (torch.tril(A @ B.T + B @ A.T + 0.5 * C0),
                        torch.tril(A.abs() @ B.abs().T + B.abs() @ A.abs().T + 0.5 * C0.abs()) + 1e-300)

        def check_err():
            Cm.copy_(C0)
            step()
            h.sync()
            ref, scale = ref_fn()
            got = torch.tril(Cm) if wl == "syr2k" else Cm
            return float(((got - ref).abs() / scale).max())
    elif wl == "tridiag":
        n = args.n if args.n != N_DEFAULT else 4096
        G = U(n, n)
        S = G + G.T
        del G
        Aw = torch.empty_like(S)
        Tw = torch.zeros(64, n, dtype=torch.float64, device="cuda")
        dw = torch.zeros(n, dtype=torch.float64, device="cuda")
        ew = torch.zeros(n - 1, dtype=torch.float64, device="cuda")
        tprec = D.PREC_OZAKI if prec == D.PREC_OZAKI else 0
        flops = 8.0 * n ** 3 / 3.0   # reduction 4/3 n^3 + forming Q 4/3 n^3
        desc = f"symmetric tridiagonal reduction + Q (T blocks of 64), {n}x{n} FP64 U[-1,1], {pname} Q formation"

        def step():
            Aw.copy_(S)
            h.sytrd(Aw, Tw, dw, ew, precision=tprec)

        def check_err():
            step()
            h.sync()
            Tr = torch.diag(dw) + torch.diag(ew, -1) + torch.diag(ew, 1)
            return float((Aw.T @ S @ Aw - Tr).abs().max() / S.abs().max())
    elif wl == "bidiag":
        n = args.n if args.n != N_DEFAULT else 4096
        A0 = U(n, n)
        Aw = torch.empty_like(A0)
        Uw = torch.empty_like(A0)
        Vw = torch.empty_like(A0)
        dw = torch.zeros(n, dtype=torch.float64, device="cuda")
        ew = torch.zeros(n - 1, dtype=torch.float64, device="cuda")
        bprec = D.PREC_OZAKI if prec == D.PREC_OZAKI else 0
        flops = 8.0 * n ** 3 / 3.0 + 4.0 * n ** 3 / 3.0 * 2   # reduction 8/3 n^3 + U and V 4/3 n^3 each
        desc = f"one-stage bidiagonal reduction + U, V, {n}x{n} FP64 U[-1,1], {pname} U/V formation"

        def step():
            Aw.copy_(A0)
            h.bidiag(Aw, dw, ew, Uw, Vw, precision=bprec)

        def check_err():
            step()
            h.sync()
            B = torch.diag(dw) + torch.diag(ew, 1)
            return float((Uw.T @ A0 @ Vw - B).abs().max() / A0.abs().max())
    elif wl == "bidiag2s":
        n = args.n if args.n != N_DEFAULT else 4096
        A0 = U(n, n)
        Aw = torch.empty_like(A0)
        Uw = torch.empty_like(A0)
        Vw = torch.empty_like(A0)
        dw = torch.zeros(n, dtype=torch.float64, device="cuda")
        ew = torch.zeros(n - 1, dtype=torch.float64, device="cuda")
        bprec = D.PREC_OZAKI if prec == D.PREC_OZAKI else 0
        # band reduction 8/3 n^3, U and V 4/3 n^3 each, back-transformation of
        # U and V by the chase's reflectors 2 n^2 (m + n) = 4 n^3 (the chase
        # itself is O(n^2) and not credited)
        flops = 8.0 * n ** 3 / 3.0 + 8.0 * n ** 3 / 3.0 + 4.0 * n ** 3
        desc = f"two-stage bidiagonal reduction (band 32, bulge chase) + U, V, {n}x{n} FP64 U[-1,1], {pname}"

        def step():
            Aw.copy_(A0)
            h.bidiag_twostage(Aw, dw, ew, Uw, Vw, precision=bprec)

        def check_err():
            step()
            h.sync()
            B = torch.diag(dw) + torch.diag(ew, 1)
            return float((Uw.T @ A0 @ Vw - B).abs().max() / A0.abs().max())
    elif wl == "einsum-chain":
        n = args.n if args.n != N_DEFAULT else 4096
        expr = "ab,bc,cd,de->ae"
        ops = [U(n, n) for _ in range(4)]
        Cm = torch.zeros(n, n, dtype=torch.float64, device="cuda")
        flops = 3 * 2.0 * n ** 3
        bytes_alg = 8.0 * 5 * n * n
        flush = L2Flush(torch, stream)
        desc = f"einsum '{expr}' (DDLA's pairwise path, intermediates on the device), all modes {n}, {pname}"

        def step():
            es.dev_einsum(h, expr, ops, Cm, precision=prec)

        def check_err():
            step()
            h.sync()
            ref = ops[0] @ ops[1] @ ops[2] @ ops[3]
            sc_ = ops[0].abs() @ ops[1].abs() @ ops[2].abs() @ ops[3].abs()
            return float(((Cm - ref).abs() / sc_).max())
    elif wl == "qr":
        n = args.n if args.n != N_DEFAULT else 8192
        A0 = U(n, n)
        Aw = torch.empty_like(A0)
        Tw = torch.zeros(min(256, n), n, dtype=torch.float64, device="cuda")
        flops = 4.0 * n ** 3 / 3.0
        qprec = D.PREC_OZAKI if prec == D.PREC_OZAKI else 0
        desc = f"Householder QR (UT-transform T blocks of 256), {n}x{n} FP64 U[-1,1], {pname} block reflectors"

        def step():
            Aw.copy_(A0)
            h.geqrf(Aw, Tw, precision=qprec)

        def check_err():
            step()
            b = U(n, 1)
            x = torch.zeros(n, 1, dtype=torch.float64, device="cuda")
            h.geqrs(Aw, Tw, b, x)
            h.sync()
            R = b - A0 @ x
            return float(R.abs().max() / (A0.abs().sum(1).max() * x.abs().max() + b.abs().max()))
    elif wl in ("einsum-a", "einsum-b"):
        if wl == "einsum-a":
            expr, sa, sb, sc = "bik,bkj->bij", (512, 256, 256), (512, 256, 256), (512, 256, 256)
            flops = 2.0 * 512 * 256 ** 3
        else:
            expr, sa, sb, sc = "abcd,cdef->abef", (64,) * 4, (64,) * 4, (64,) * 4
            flops = 2.0 * 64 ** 6
        A, B = U(*sa), U(*sb)
        Cm = torch.zeros(*sc, dtype=torch.float64, device="cuda")
        bytes_alg = 8.0 * (A.numel() + B.numel() + 2 * Cm.numel())
        d = es.plan(expr, np.empty(sa), np.empty(sb), np.empty(sc))
        Le = es._declare()
        flush = L2Flush(torch, stream)
        desc = f"einsum '{expr}' {sa} x {sb}, FP64 U[-1,1], {pname}"

        def step():
            D._lib.check(Le.ddla_dev_contract(h.h, C.byref(d), 1.0, C.c_void_p(A.data_ptr()),
                                              C.c_void_p(B.data_ptr()), C.c_void_p(Cm.data_ptr()), prec), "contract")

        def check_err():
            Cm.zero_()
            step()
            h.sync()
            ref = torch.einsum(expr, A, B)
            sc_ = torch.einsum(expr, A.abs(), B.abs())
            return float(((Cm - ref).abs() / sc_).max())
    elif wl == "chol":
        n, nrhs = args.n if args.n != N_DEFAULT else 16384, 16
        G = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
        A = torch.eye(n, dtype=torch.float64, device="cuda")
        h.gemm(1.0 / n, G, G, 1.0, A, tb=D.TRANSPOSE, precision=D.PREC_OZAKI)   # A = G G^T / n + I
        h.sync()
        del G
        A = 0.5 * (A + A.T)   # exactly symmetric
        b = torch.randn(n, nrhs, dtype=torch.float64, device="cuda", generator=g)
        X = torch.zeros(n, nrhs, dtype=torch.float64, device="cuda")
        flops = n ** 3 / 3.0 + 2.0 * n * n * nrhs
        desc = f"Cholesky + solve, SPD G G^T/n + I, n={n}, {nrhs} RHS, {pname}"
        if prec == D.PREC_FP64:
            F = torch.empty_like(A)

            def step():
                F.copy_(A)
                rc = h.potrf(D.LOWER, F)
                if rc != 0:
                    raise RuntimeError(f"potrf failed {rc}")
                X.copy_(b)
                h.potrs(D.LOWER, F, X)
        else:
            def step():
                rc, rep = h.gesv_mixed(A, b, X, precision=prec, tol=TOL, spd=True)
                if rc != 0 or not rep["converged"]:
                    raise RuntimeError(f"posv_mixed failed rc={rc} rep={rep}")
                last_rep.update(rep)

        def check_err():
            step()
            h.sync()
            R = b - A @ X
            an = A.abs().sum(1).max()
            return float((R.abs().amax(0) / (an * X.abs().amax(0) + b.abs().amax(0))).max())
    elif wl == "batched":
        r = np.random.default_rng(SEED + 4)
        count = 20000
        sizes = r.integers(8, 257, count)
        kinds = np.where(np.arange(count) % 2 == 0, 0, 2)
        mats, rhs = [], []
        for nn, k in zip(sizes, kinds):
            if k == 2:
                Gs = r.standard_normal((nn, nn))
                mats.append(Gs @ Gs.T / nn + np.eye(nn))
            else:
                mats.append(r.standard_normal((nn, nn)) + nn * np.eye(nn))
            rhs.append(r.standard_normal(nn))
        mixed = prec != D.PREC_FP64
        bs = bt.BatchedSolver(h, sizes, kinds, mixed=mixed, tol=TOL if mixed else 0.0)
        bs.load(mats, rhs)
        s3 = sizes.astype(np.float64)
        flops = float(np.sum(np.where(kinds == 0, 2.0 / 3.0, 1.0 / 3.0) * s3 ** 3 + 2.0 * s3 ** 2))
        bytes_alg = float(2 * 8 * np.sum(s3 ** 2))
        desc = f"batched {count} solves (half PLU of N(0,1)+nI, half Cholesky of G G^T/n+I), n ~ U{{8..256}}, " + \
            ("mixed fp32 + FP64 refinement" if mixed else "fp64")

        def step():
            bs.reset()
            bs.run()

        def check_err():
            step()
            res, info, iters = bs.results()
            worst = 0.0
            for i in range(0, count, 97):
                x = res[i][1]
                A0 = mats[i]
                rr = rhs[i] - A0 @ x
                worst = max(worst, np.abs(rr).max() / (np.abs(A0).sum(1).max() * np.abs(x).max() +
                                                       np.abs(rhs[i]).max()))
            return worst
    else:
        raise SystemExit(f"unknown workload {wl}")

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    launches0 = D.kernel_launches()
    clocks.start()
    times = []
    for _ in range(args.steps):
        if flush is not None:
            flush()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    launches = D.kernel_launches() - launches0
    ms = statistics.median(times)
    value = flops / (ms * 1e-3) / 1e9
    classes = None
    if wl in ("qr", "tridiag", "bidiag", "bidiag2s"):
        # one more step with per-class CUDA-event brackets (outside the timed steps)
        L.ddla_timing_enable(1)
        step()
        torch.cuda.synchronize()
        classes = {}
        names = {1: "qr_panel", 7: "qr_t_factor", 0: "block_reflector_gemm", 2: "trsm"} if wl == "qr" else \
            {9: "band_reduction_and_uv", 10: "bulge_chase", 11: "back_transformation",
             0: "block_reflector_gemm"} if wl == "bidiag2s" else {1: "reduction", 0: "form_q"}
        for cls, name in names.items():
            t_ms, cnt, fl, by = C.c_double(), C.c_int64(), C.c_double(), C.c_double()
            L.ddla_timing_read(cls, C.byref(t_ms), C.byref(cnt), C.byref(fl), C.byref(by))
            classes[name] = {"ms": t_ms.value, "launches": cnt.value,
                             "gflops": fl.value / (t_ms.value * 1e-3) / 1e9 if t_ms.value else 0.0}
        L.ddla_timing_enable(0)
    err = check_err() if check_err else None
    f64_peak, f32_peak = dv.measure_peaks()
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    if prec == D.PREC_FP64:
        roof = {"bound": "tensor", "achieved": value / 1e3, "peak": f64_peak, "unit": "TFLOP/s",
                "frac": value / 1e3 / f64_peak, "peak_source": "live DMMA probe (ddla_measure_peaks)"}
    elif prec == D.PREC_OZAKI:
        roof = {"bound": "tensor", "achieved": value / 1e3, "peak": peaks.get("bf16_tflops", 1900.0) / 36.0,
                "unit": "TFLOP/s (FP64-equivalent)", "peak_source": "MEASURED_PEAKS.json bf16_tflops / 36 slice "
                "products (8 slices, levels 0..7)"}
        roof["frac"] = roof["achieved"] / roof["peak"]
    else:
        roof = {"bound": "fp32-cuda-core", "achieved": value / 1e3, "peak": f32_peak, "unit": "TFLOP/s",
                "frac": value / 1e3 / f32_peak, "peak_source": "live FFMA probe (ddla_measure_peaks)"}
    roof["traffic"] = None
    roof["note"] = "whole-step algorithmic flops / median CUDA-event step time"
    if bytes_alg:
        roof["hbm_gbs"] = bytes_alg / (ms * 1e-3) / 1e9
    out = {"metric": f"{wl} GFLOP/s", "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": pname, "data": "synthetic, seeded",
           "config": {"workload": desc, "precision": pname,
                      "l2": "L2 flushed between steps" if flush else "inputs larger than L2"},
           "error": err, "roofline": roof, "gpu_launches": launches, "clocks": clk, "classes": classes,
           "solve_report": {k: last_rep[k] for k in ("iterations", "factor_ms", "refine_ms") if k in last_rep} or None,
           "peaks_live": {"fp64_tflops": f64_peak, "fp32_tflops": f32_peak}}
    print(json.dumps(out))
    h.close()


def timed_steps(step, steps, warmup, stream, torch):
    """Run `warmup` untimed steps, then time `steps` with CUDA events on the
    solve stream (device synchronised on both sides); ms per step."""
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def gpu_berr(A, X, b):
    """max ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), FP64 on the
    device (torch), outside every timed region."""
    R = b - A @ X
    return float((R.abs().amax() / (A.abs().sum(1).amax() * X.abs().amax() + b.abs().amax())).item())


def rel_inf(x, ref):
    return float(((x - ref).abs().max() / ref.abs().max()).item())


def lu_pair(h, D, torch, A, b, prec, steps, warmup, stream, piv_out=None):
    """The mixed solve and the plain FP64 LU + solve on the same A and b.
    Returns (mixed ms, plain ms, dict of accuracy figures)."""
    n = A.shape[0]
    X = torch.zeros(n, 1, dtype=torch.float64, device="cuda")
    X64 = torch.zeros_like(X)
    F = torch.empty_like(A)
    piv64 = torch.zeros(n, dtype=torch.int32, device="cuda")

    def plain():
        F.copy_(A)
        rc = h.getrf(F, piv64)
        if rc != 0:
            raise RuntimeError(f"getrf failed rc={rc} err={D._lib.last_error()}")
        X64.copy_(b)
        h.getrs(F, piv64, X64)

    reps = []

    def mixed():
        rc, rep = h.gesv_mixed(A, b, X, precision=prec, tol=TOL)
        if rc != 0 or not rep["converged"]:
            raise RuntimeError(f"solve failed rc={rc} rep={rep} err={D._lib.last_error()}")
        reps.append(rep)

    ms_plain = timed_steps(plain, steps[1], warmup[1], stream, torch)
    ms_mixed = timed_steps(mixed, steps[0], warmup[0], stream, torch)
    # one more mixed solve, untimed, that also compares its pivots with the
    # FP64 ones and its solution with the FP64 solution
    pv = piv_out if piv_out is not None else torch.zeros(n, dtype=torch.int32, device="cuda")
    rc, rep = h.gesv_mixed(A, b, X, x_ref=X64, precision=prec, tol=TOL, piv_ref=piv64, piv_out=pv)
    if rc != 0:
        raise RuntimeError(f"solve failed rc={rc}")
    acc = {"mixed_backward_error": gpu_berr(A, X, b), "plain_backward_error": gpu_berr(A, X64, b),
           "mixed_vs_plain_forward_error": rep["forward_error"],
           "pivots_agree": rep["pivots_agree"], "pivots_first_diff": rep["pivots_first_diff"],
           "refine_iterations": reps[-1]["iterations"], "factor_ms": reps[-1]["factor_ms"],
           "refine_ms": reps[-1]["refine_ms"], "library_backward_error": reps[-1]["backward_error"]}
    return ms_mixed, ms_plain, acc, X, X64, piv64


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--precision", default="auto", choices=["auto", "fp32", "tf32x3", "bf16x3", "fp64", "ozaki"])
    ap.add_argument("--tune", action="append", default=[], metavar="KEY=VALUE",
                    help="library tuning key (ddla_tune_set) applied before the run; repeatable")
    ap.add_argument("--workload", default="lu", choices=["lu", "gemm", "chol", "batched", "einsum-a", "einsum-b",
                                                         "symm", "trmm", "syr2k", "qr", "einsum-chain",
                                                         "tridiag", "bidiag", "bidiag2s"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the oracle (CPU baseline and its checks)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-big", action="store_true", help="skip the n = 16384 sub-record")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload != "lu":
        return secondary(args)

    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    import ddla_gb300 as D
    from ddla_gb300 import device as dv
    from ddla_gb300 import build as bld
    bld.build()
    L = D.lib()
    apply_tune(args)

    prec_map = {"fp32": D.PREC_FP32, "tf32x3": D.PREC_TF32X3, "bf16x3": D.PREC_BF16X3}
    prec_name = args.precision if args.precision not in ("auto", "fp64", "ozaki") else "tf32x3"
    prec = prec_map[prec_name]
    n = args.n
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    h = dv.Handle(stream)
    Ah, bh = headline_inputs(n, SEED + rank)
    A = torch.from_numpy(Ah).cuda()
    b = torch.from_numpy(bh).cuda()
    X = torch.zeros(n, 1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()

    def step():
        rc, rep = h.gesv_mixed(A, b, X, precision=prec, tol=TOL)
        if rc != 0 or not rep["converged"]:
            raise RuntimeError(f"solve failed rc={rc} rep={rep} err={D._lib.last_error()}")
        return rep

    for _ in range(args.warmup):
        step()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local)
    L.ddla_timing_enable(1)
    launches0 = D.kernel_launches()
    barrier()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    reps = [step() for _ in range(args.steps)]
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    launches = D.kernel_launches() - launches0
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world)
    value = replica_value(lu_flops(n), world, ms)

    # dominant kernel class from the per-launch CUDA-event records of the timed region
    classes = {0: "trailing_update_gemm", 1: "lu_panel", 2: "trsm", 3: "laswp", 4: "refinement_residual",
               8: "refinement_solves"}
    per = {}
    for cls in classes:
        t_ms, cnt, fl, by = C.c_double(), C.c_int64(), C.c_double(), C.c_double()
        L.ddla_timing_read(cls, C.byref(t_ms), C.byref(cnt), C.byref(fl), C.byref(by))
        per[classes[cls]] = {"ms_per_step": t_ms.value / args.steps, "launches": cnt.value, "flops": fl.value,
                             "bytes": by.value}
    L.ddla_timing_enable(0)
    f64_peak, f32_peak = dv.measure_peaks()
    dom = max(("trailing_update_gemm", "lu_panel"), key=lambda k: per[k]["ms_per_step"])
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    hbm_src = "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback 6.8 TB/s (of fallback)"

    def hbm_entry(cls, kernel, traffic, note):
        v = per[cls]
        nl = max(v["launches"], 1)
        ms_launch = v["ms_per_step"] * args.steps / nl
        gbs = (v["bytes"] / nl) / (ms_launch * 1e-3) / 1e9 if v["launches"] else 0.0
        tfs = (v["flops"] / nl) / (ms_launch * 1e-3) / 1e12 if v["launches"] else 0.0
        return {"bound": "hbm", "kernel": kernel, "achieved": gbs, "peak": hbm, "unit": "GB/s",
                "frac": gbs / hbm if hbm else None, "traffic": traffic, "peak_source": hbm_src,
                "launches_per_step": v["launches"] / args.steps, "us_per_launch": ms_launch * 1e3,
                "algorithmic_bytes_per_launch": v["bytes"] / nl, "tflops": tfs, "note": note}

    upd_kernel = {D.PREC_TF32X3: "k_tc_update (tcgen05 3xTF32, persistent)",
                  D.PREC_BF16X3: "k_tc_update (tcgen05 3xBF16, persistent)"}.get(prec, "k_supdate (FP32 CUDA cores)")
    # DRAM bytes of one launch from the ncu captures summarised in profiles/
    roof_panel = hbm_entry("lu_panel", "k_panel_lu (LU panel, 16-CTA cluster)", PANEL_TRAFFIC,
                           "latency-bound: one candidate exchange per column; algorithmic bytes = the panel read "
                           "and written once (2 m w 4 B)")
    roof_update = hbm_entry("trailing_update_gemm", upd_kernel, None,
                            "rank-64 update C -= L21 U12: algorithmic bytes = C read + written + the two panels; "
                            "tflops = 2 m n k per launch over its duration")
    roofline = dict(roof_panel if dom == "lu_panel" else roof_update)
    roofline["dominant_class"] = dom
    roofline["classes_ms_per_step"] = {k: round(v["ms_per_step"], 4) for k, v in per.items()}
    roofline["other"] = roof_update if dom == "lu_panel" else roof_panel

    # end-to-end through the host C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e and rank == 0:
        Ahp = torch.from_numpy(Ah).pin_memory()
        bhp = torch.from_numpy(bh).pin_memory()
        xh = torch.zeros(n, 1, dtype=torch.float64).pin_memory()
        opts = D._lib.Opts()
        opts.precision, opts.tol = prec, TOL
        rep = D._lib.SolveReport()

        def e2e_step():
            rc = L.ddla_dgesv_mixed(n, 1, C.c_void_p(Ahp.data_ptr()), n, 1, C.c_void_p(bhp.data_ptr()), 1, 1,
                                    C.c_void_p(xh.data_ptr()), 1, 1, None, C.byref(opts), C.byref(rep))
            if rc != 0:
                raise RuntimeError(f"e2e solve failed {rc}: {D._lib.last_error()}")
        for _ in range(3):
            e2e_step()
        k2 = max(3, min(args.steps, 5))
        t = time.perf_counter()
        for _ in range(k2):
            e2e_step()
        dt = (time.perf_counter() - t) / k2
        e2e = {"value": lu_flops(n) / dt / 1e9, "unit": UNIT, "ms_per_step": dt * 1e3,
               "h2d_bytes_per_step": n * n * 8 + n * 8, "d2h_bytes_per_step": n * 8,
               "api": "ddla_dgesv_mixed (host pointers, synchronous)"}

    # the plain FP64 GPU path on the same A and b (the metric's comparison),
    # and the accuracy figures of both
    ms_m2, ms_plain, acc, Xm, X64, piv64 = lu_pair(h, D, torch, A, b, prec, (3, 3), (3, 3), stream)
    plain = {"ms_per_step": ms_plain, "value": lu_flops(n) / (ms_plain * 1e-3) / 1e9, "unit": UNIT,
             "backward_error": acc["plain_backward_error"],
             "path": "ddla_dev_dgetrf + ddla_dev_dgetrs: FP64 LU with partial pivoting (DMMA trailing updates, "
                     "cluster panels) and FP64 triangular solves, on a fresh copy of A each step",
             "steps": 3, "warmup": 3}

    # CPU baseline on the same system (rank 0, one GPU): the oracle, which also
    # checks the pivots of the FP64 GPU path and gives an independent FP64
    # solution for the forward errors
    cpu = None
    oracle_check = None
    if not args.no_cpu and rank == 0 and world == 1:
        threads = max(1, (os.cpu_count() or 2) // 2)
        Fo, po, xo, dt = oracle_solve(Ah, bh, threads)
        cpu = {"value": lu_flops(n) / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"oracle dgetrf+dgetrs (C restatement of DDLA's managed LU) on the same n={n} system, one "
                         f"solve, {dt:.2f} s, ProcessorCount/2 threads like ParallelHelperEX"}
        xo_t = torch.from_numpy(xo).cuda()
        p64 = piv64.cpu().numpy()
        diff = np.nonzero(p64 != po)[0]
        oracle_check = {"plain_pivots_identical": bool(diff.size == 0),
                        "plain_pivots_first_diff": int(diff[0]) if diff.size else -1,
                        "mixed_pivots_agree_with_oracle": None,
                        "plain_forward_error_vs_oracle": rel_inf(X64, xo_t),
                        "mixed_forward_error_vs_oracle": rel_inf(Xm, xo_t),
                        "oracle_backward_error": float(np.max(np.abs(bh - Ah @ xo)) /
                                                       (np.abs(Ah).sum(1).max() * np.abs(xo).max() +
                                                        np.abs(bh).max()))}
        po_d = torch.from_numpy(po.astype(np.int32)).cuda()
        rc, rep = h.gesv_mixed(A, b, X, x_ref=xo_t, precision=prec, tol=TOL, piv_ref=po_d)
        oracle_check["mixed_pivots_agree_with_oracle"] = rep["pivots_agree"]
        oracle_check["mixed_pivots_first_diff_vs_oracle"] = rep["pivots_first_diff"]

    # the spec size: n = 16384, mixed and plain FP64 (a few steps each)
    big = None
    if not args.no_big and rank == 0:
        del Xm, X64
        nb_ = 16384
        g = torch.Generator(device="cuda").manual_seed(SEED + 16384)
        Ab = torch.randn(nb_, nb_, dtype=torch.float64, device="cuda", generator=g)
        bb = torch.randn(nb_, 1, dtype=torch.float64, device="cuda", generator=g)
        msb, msb_plain, accb, _, _, _ = lu_pair(h, D, torch, Ab, bb, prec, (5, 2), (3, 1), stream)
        big = {"n": nb_, "data": "A, b i.i.d. N(0,1) (seeded device generator)",
               "mixed": {"ms_per_step": msb, "value": lu_flops(nb_) / (msb * 1e-3) / 1e9, "steps": 5, "warmup": 3},
               "plain_fp64": {"ms_per_step": msb_plain, "value": lu_flops(nb_) / (msb_plain * 1e-3) / 1e9,
                              "steps": 2, "warmup": 1},
               "vs_plain_fp64": msb_plain / msb, **accb}
        del Ab, bb
        torch.cuda.empty_cache()

    if rank == 0:
        last = reps[-1]
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None,
               "dtype": {D.PREC_TF32X3: "f32 factor with 3xTF32 tensor-core updates + f64 refinement",
                         D.PREC_BF16X3: "f32 factor with 3xBF16 tensor-core updates + f64 refinement"}.get(
                             prec, "f32 factor + f64 refinement"),
               "data": "synthetic N(0,1), seeded host generator, inputs 512 MB > L2 (no flush needed)",
               "config": headline_config(n, world),
               "method": f"mixed {prec_name} factor + FP64 refinement (flexible GMRES preconditioned by the "
                         f"factors)",
               "plain_fp64": plain, "vs_plain_fp64": ms_plain / ms,
               "backward_error": last["backward_error"], "refine_iterations": last["iterations"],
               "factor_ms": last["factor_ms"], "refine_ms": last["refine_ms"], "accuracy": acc,
               "oracle_check": oracle_check, "n16384": big,
               "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
               "clocks": clk, "peaks_live": {"fp64_tflops": f64_peak, "fp32_tflops": f32_peak}}
        print(json.dumps(out))
    h.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
