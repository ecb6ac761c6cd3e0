"""GPU: the autotuner on a small uneven batch.  Every candidate plan must
solve correctly, the winner is one of the candidates, and the solver built
with the winning table still meets the FP64 backward-error target."""
import numpy as np
import pytest

from helpers import berr, rng, spd

pytestmark = pytest.mark.gpu


def test_tune_batched_small(ddla):
    from ddla_gb300 import autotune, batched, device
    r = rng(91)
    sizes = list(r.integers(8, 200, 120))
    kinds = [0 if i % 2 == 0 else 2 for i in range(len(sizes))]
    mats = [spd(r, n) if k == 2 else r.standard_normal((n, n)) + n * np.eye(n) for n, k in zip(sizes, kinds)]
    rhs = [r.standard_normal(n) for n in sizes]
    grid = {"batched.nb.big": [16, 32], "batched.ctas_per_sm": [1, 2]}
    try:
        best, t, log = autotune.tune_batched(sizes, kinds, mats, rhs, mixed=True, grid=grid, reps=2)
        assert best in [c for c, _ in log] and t == min(tt for _, tt in log) and t > 0
        autotune.apply(best)
        h = device.Handle()
        bs = batched.BatchedSolver(h, sizes, kinds, mixed=True, tol=1e-14)
        bs.load(mats, rhs)
        bs.run()
        res, info, iters = bs.results()
        bs.close()
        h.close()
        assert np.all(info == 0)
        for (F, x, piv), A, b in zip(res, mats, rhs):
            assert berr(A, x, b) <= 1e-14
    finally:
        for k in grid:
            autotune.tune_set(k, 0)
