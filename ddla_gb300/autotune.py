"""Autotuner for the tuning keys of libddla_gb300 (no learned component).

Tuning keys (read by the library through ddla_tune_get at plan / call time):
  lu.nb                   LU panel width cap (0 = automatic: 64 FP32 / 32 FP64)
  lu.lookahead            1 = factor panel k+1 on a side stream during update k
  panel.cluster           cluster size cap of the LU panel kernel
  batched.nb.<bucket>     panel width of the batched kernel per size bucket
                          (bucket 32 / 64 / 128 / big by matrix order)
  batched.ctas_per_sm     resident CTAs per SM of the persistent batched kernel

The search is coordinate descent over small candidate grids: each key in turn
takes the candidate with the lowest median device time (CUDA events over
`reps` runs of the caller's own workload) while the others hold their best
values.  The winners form a JSON table that `load` applies with ddla_tune_set.

    python -m ddla_gb300.autotune --solve 8192 --out tune.json
    python -m ddla_gb300.autotune --batched 2000 --out tune.json
"""
import argparse
import json
import statistics

from ._lib import check, lib

# The first candidate of every key is the library's automatic choice (0, or 1
# for lu.lookahead, which is on unless set to 0): the search starts from the
# defaults and only moves when a candidate is faster.
SOLVE_GRID = {"lu.nb": [0, 32, 16], "panel.cluster": [0, 8], "lu.lookahead": [1, 0]}
BATCHED_GRID = {"batched.nb.32": [0, 4, 16, 32], "batched.nb.64": [0, 8, 32], "batched.nb.128": [0, 16],
                "batched.nb.big": [0, 16], "batched.ctas_per_sm": [0, 1, 2]}


def tune_set(key, value):
    check(lib().ddla_tune_set(key.encode(), int(value)), f"tune_set {key}")


def tune_get(key, dflt=0):
    return int(lib().ddla_tune_get(key.encode(), int(dflt)))


def apply(table):
    for k, v in table.items():
        tune_set(k, v)


def save(table, path):
    with open(path, "w") as f:
        json.dump(dict(sorted(table.items())), f, indent=1)


def load(path):
    """Reads a table written by `save` and applies it; returns it."""
    with open(path) as f:
        table = {k: int(v) for k, v in json.load(f).items()}
    apply(table)
    return table


def search(grid, time_fn, start=None, sweeps=1):
    """Coordinate descent.  time_fn(table) -> seconds (lower is better) is
    called with the full candidate table; returns (best table, best time, log)."""
    best = dict(start or {k: v[0] for k, v in grid.items()})
    best_t = time_fn(dict(best))
    log = [(dict(best), best_t)]
    for _ in range(sweeps):
        for key, cands in grid.items():
            for v in cands:
                if v == best[key]:
                    continue
                cand = dict(best)
                cand[key] = v
                t = time_fn(cand)
                log.append((cand, t))
                if t < best_t:
                    best, best_t = cand, t
    return best, best_t, log


def _timer(torch, stream, fn, reps):
    times = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    return statistics.median(times)


def tune_solve(n, precision=1, grid=None, reps=3, seed=0):
    """Tunes the mixed LU solve (ddla_dev_dgesv_mixed) on an n x n N(0,1) system."""
    import torch
    from .device import Handle
    stream = torch.cuda.Stream()
    h = Handle(stream)
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    b = torch.randn(n, 1, dtype=torch.float64, device="cuda", generator=g)
    X = torch.zeros_like(b)
    torch.cuda.synchronize()

    def run():
        rc, rep = h.gesv_mixed(A, b, X, precision=precision, tol=1e-14)
        check(rc, "gesv_mixed")
        if not rep["converged"]:
            raise RuntimeError("tuning solve did not converge")

    def time_fn(table):
        apply(table)
        run()   # warm-up (workspaces, graph of the side stream)
        return _timer(torch, stream, run, reps)

    try:
        return search(grid or SOLVE_GRID, time_fn)
    finally:
        h.close()


def tune_batched(sizes, kinds, mats, rhs, mixed=True, grid=None, reps=3):
    """Tunes the batched plan on the caller's own items (a plan is rebuilt
    for every candidate since the keys are read at plan creation)."""
    import torch
    from .batched import BatchedSolver
    from .device import Handle
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    h = Handle(stream)

    def time_fn(table):
        apply(table)
        bs = BatchedSolver(h, sizes, kinds, mixed=mixed, tol=1e-14 if mixed else 0.0)
        try:
            bs.load(mats, rhs)

            def run():
                bs.reset()
                bs.run()
            run()
            return _timer(torch, stream, run, reps)
        finally:
            bs.close()

    try:
        return search(grid or BATCHED_GRID, time_fn)
    finally:
        h.close()


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--solve", type=int, default=0, help="tune the mixed LU solve at this n")
    ap.add_argument("--batched", type=int, default=0, help="tune a batch of this many uneven items")
    ap.add_argument("--out", default="ddla_tune.json")
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    table = {}
    if a.solve:
        best, t, _ = tune_solve(a.solve, reps=a.reps)
        print(f"solve n={a.solve}: {t * 1e3:.2f} ms with {best}")
        table.update(best)
    if a.batched:
        import numpy as np
        r = np.random.default_rng(4)
        sizes = r.integers(8, 257, a.batched)
        kinds = np.where(np.arange(a.batched) % 2 == 0, 0, 2)
        mats, rhs = [], []
        for nn, k in zip(sizes, kinds):
            if k == 2:
                G = r.standard_normal((nn, nn))
                mats.append(G @ G.T / nn + np.eye(nn))
            else:
                mats.append(r.standard_normal((nn, nn)) + nn * np.eye(nn))
            rhs.append(r.standard_normal(nn))
        best, t, _ = tune_batched(sizes, kinds, mats, rhs, reps=a.reps)
        print(f"batched {a.batched}: {t * 1e3:.2f} ms with {best}")
        table.update(best)
    save(table, a.out)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
