"""GPU: batched uneven factorizations in one persistent launch against the
oracle (per-item factors, pivots, solutions) and the mixed FP32 + FP64
refinement path against the FP64 backward-error target."""
import numpy as np
import pytest

from helpers import berr, rel_max, rng, spd

pytestmark = pytest.mark.gpu


def _items(r, sizes, kinds):
    mats, rhs = [], []
    for n, k in zip(sizes, kinds):
        if k == 2:
            mats.append(spd(r, n))
        elif k == 1:
            mats.append(r.standard_normal((n, n)) + n * np.eye(n))
        else:
            mats.append(r.standard_normal((n, n)) + (n * np.eye(n) if r.random() < 0.5 else 0))
        rhs.append(r.standard_normal(n))
    return mats, rhs


@pytest.fixture(scope="module")
def handle(ddla):
    from ddla_gb300 import device
    h = device.Handle()
    yield h
    h.close()


def test_batched_plain_matches_oracle(ddla, orc, handle):
    from ddla_gb300 import batched
    r = rng(11)
    sizes = [1, 2, 7, 8, 31, 32, 33, 64, 65, 100, 128, 129, 200, 256] * 3
    kinds = [i % 3 for i in range(len(sizes))]
    mats, rhs = _items(r, sizes, kinds)
    bs = batched.BatchedSolver(handle, sizes, kinds, mixed=False)
    bs.load(mats, rhs)
    bs.run()
    res, info, iters = bs.results()
    assert np.all(info == 0)
    for (F, x, piv), A, b, k in zip(res, mats, rhs, kinds):
        Fo = A.copy()
        if k == 0:
            rc, po = orc.dgetrf(Fo)
            assert np.array_equal(piv, po)
            assert rel_max(F, Fo) <= 1e-10
        elif k == 1:
            orc.dgetrf_nopiv(Fo)
            assert rel_max(F, Fo) <= 1e-11
        else:
            orc.dpotrf(0xC0, Fo)
            assert rel_max(np.tril(F), np.tril(Fo)) <= 1e-12
        assert berr(A, x, b) <= 1e-14
    bs.close()


def test_batched_mixed_refines_to_fp64(ddla, handle):
    from ddla_gb300 import batched
    r = rng(12)
    sizes = list(r.integers(8, 257, size=120))
    kinds = [0 if i % 2 == 0 else 2 for i in range(len(sizes))]
    mats, rhs = _items(r, sizes, kinds)
    bs = batched.BatchedSolver(handle, sizes, kinds, mixed=True)
    bs.load(mats, rhs)
    for _ in range(2):     # graph replay
        bs.run()
    res, info, iters = bs.results()
    assert np.all(info == 0)
    assert np.all(iters >= 0), iters
    for (_, x, _), A, b in zip(res, mats, rhs):
        assert berr(A, x, b) <= 1e-14
    bs.close()


def test_batched_failures_per_item(ddla, orc, handle):
    from ddla_gb300 import batched
    A1 = np.eye(40)
    A1[10, 10] = -1.0                      # indefinite for Cholesky
    A2 = np.eye(50)
    A2[:, 7] = 0.0                          # singular for LU
    A3 = np.eye(30) * 2.0
    mats, rhs = [A1, A2, A3], [np.ones(40), np.ones(50), np.ones(30)]
    bs = batched.BatchedSolver(handle, [40, 50, 30], [2, 0, 0], mixed=False)
    bs.load(mats, rhs)
    bs.run()
    res, info, _ = bs.results()
    assert info[0] == orc.dpotrf(0xC0, A1.copy()) == 11
    assert info[1] == orc.dgetrf(A2.copy())[0] == 8
    assert info[2] == 0
    assert np.allclose(res[2][1], 0.5)
    bs.close()
