"""The split triangular solve's protocol finishes and gives the sequential
result under any interleaving and any residency of its CTAs.

The one-right-hand-side solve (trsm.cu, k_trsv_cluster in split mode) runs
the dependency chain on one 16-CTA cluster and streams the far tiles on
helper CTAs (DDLA's managed solve is the plain block forward substitution,
DDLA/BLAS/Managed/3m/TrSM.cs:62-122).  The roles and the rows are taken with
atomics:
  * the first cluster to start becomes the chain (atomicCAS on a role word);
  * helpers take block rows l > W in increasing order from a counter and
    claim each with atomicCAS(rowst[l], 0 -> 2); the chain claims row l with
    atomicCAS(rowst[l], 0 -> 1) when it reaches it and then sums the far
    tiles itself;
  * a helper waits for flag[j] (x_j published) before each far tile, then
    stores the far sum and sets rowst[l] = 3; the chain waits for rowst[l] == 3
    at its near tile l - PW; every block ends with x_l = inv(A_ll) acc -
    M_l x_{l-1}.
This test replays that protocol as coroutines, one per CTA, under random
interleavings and with the clusters admitted one at a time or a few at a
time in random order (a cluster that has not started cannot be waited for),
with W, PW and the clamp read from the source.  It checks that no run
deadlocks, that every far sum is formed exactly once, and that x equals the
sequential block solve.
"""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "ddla_gb300", "csrc", "trsm.cu")


def _defaults():
    src = open(SRC).read()
    w = int(re.search(r'tune_get\("trsv\.split\.w",\s*(\d+)\)', src).group(1))
    pw = int(re.search(r'tune_get\("trsv\.split\.pw",\s*(\d+)\)', src).group(1))
    # fused mode: the near window's last tile is folded into M_l, so PW >= 2
    assert "const int pmin = mlast ? 2 : 1;" in src
    return w, pw


def _system(nblk, tb, seed):
    r = np.random.default_rng(seed)
    n = nblk * tb
    L = np.tril(r.uniform(-1, 1, (n, n)) / n) + 2 * np.eye(n)
    b = r.standard_normal(n)
    return L, b


class _Run:
    def __init__(self, L, b, nblk, tb, cs, W, PW, groups, capacity, seed):
        self.L, self.b, self.nblk, self.tb = L, b, nblk, tb
        self.cs, self.W, self.PW = cs, W, PW
        self.rng = np.random.default_rng(seed)
        self.xflag = [0] * nblk
        self.rowst = [0] * nblk
        self.next = 0
        self.role = 0
        self.X = np.zeros(nblk * tb)
        self.part = np.zeros(nblk * tb)
        self.far_sums = [0] * nblk   # how many times row l's far sum was formed
        self.groups, self.capacity = groups, capacity

    def blk(self, i, j):
        t = self.tb
        return self.L[i * t:(i + 1) * t, j * t:(j + 1) * t]

    def chain(self, rank):
        W, PW, t = self.W, self.PW, self.tb
        for l in range(rank, self.nblk, self.cs):
            helped = l > W
            own = False
            if helped:
                own = self.rowst[l] == 0
                if own:
                    self.rowst[l] = 1
            acc = self.b[l * t:(l + 1) * t].copy()
            if helped and own:
                for j in range(0, l - W):
                    yield lambda j=j: self.xflag[j]
                    acc -= self.blk(l, j) @ self.X[j * t:(j + 1) * t]
                self.far_sums[l] += 1
            jlo = l - W if helped else 0
            for j in range(jlo, l - 1):   # the last tile is folded into M_l
                yield lambda j=j: self.xflag[j]
                acc -= self.blk(l, j) @ self.X[j * t:(j + 1) * t]
                if helped and not own and j == l - PW:
                    yield lambda: self.rowst[l] == 3
                    acc -= self.part[l * t:(l + 1) * t]
            y = np.linalg.solve(self.blk(l, l), acc)
            if l > 0:
                yield lambda: self.xflag[l - 1]
                M = np.linalg.solve(self.blk(l, l), self.blk(l, l - 1))
                y = y - M @ self.X[(l - 1) * t:l * t]
            self.X[l * t:(l + 1) * t] = y
            self.xflag[l] = 1

    def helper(self):
        W, t = self.W, self.tb
        while True:
            row = self.next + W + 1
            self.next += 1
            if row >= self.nblk:
                return
            if self.rowst[row] != 0:
                continue
            self.rowst[row] = 2
            f = np.zeros(t)
            for j in range(0, row - W):
                yield lambda j=j: self.xflag[j]
                f += self.blk(row, j) @ self.X[j * t:(j + 1) * t]
            self.part[row * t:(row + 1) * t] = f
            self.far_sums[row] += 1
            self.rowst[row] = 3
            yield lambda: True

    def run(self):
        """Clusters are admitted in random order, `capacity` at a time; the
        first one admitted takes the chain role.  Each step advances one
        random CTA whose wait is satisfied."""
        order = list(self.rng.permutation(self.groups))
        resident, live = [], {}
        steps = 0
        while True:
            while order and len(resident) < self.capacity:
                g = order.pop(0)
                if self.role == 0:
                    self.role = g + 1
                    ctas = [self.chain(r) for r in range(self.cs)]
                else:
                    ctas = [self.helper() for _ in range(self.cs)]
                live[g] = [[c, lambda: True] for c in ctas]
                resident.append(g)
            ready = [(g, i) for g in resident for i, (c, w) in enumerate(live[g]) if c is not None and w()]
            if not ready:
                busy = [g for g in resident if any(c is not None for c, _ in live[g])]
                assert not busy, "deadlock: every resident CTA waits"
                resident = [g for g in resident if g in busy]
                if not order:
                    return
                continue
            g, i = ready[self.rng.integers(len(ready))]
            c = live[g][i][0]
            try:
                live[g][i][1] = next(c)
            except StopIteration:
                live[g][i][0] = None
            if all(cc is None for cc, _ in live[g]):
                resident.remove(g)
            steps += 1
            assert steps < 10 ** 6


@pytest.mark.parametrize("nblk,groups,capacity", [(20, 3, 3), (40, 4, 2), (40, 8, 8), (64, 5, 1), (33, 2, 2),
                                                  (17, 4, 4), (18, 2, 1)])
def test_split_schedule_finishes_with_the_sequential_result(nblk, groups, capacity):
    W, PW = _defaults()
    tb, cs = 3, 4   # small blocks and a 4-CTA cluster keep the replay short
    for seed in range(6):
        L, b = _system(nblk, tb, seed)
        run = _Run(L, b, nblk, tb, cs, W, PW, groups, capacity, seed)
        run.run()
        x_ref = np.linalg.solve(L, b)
        assert np.allclose(run.X, x_ref, rtol=1e-10, atol=1e-12)
        assert all(f == (1 if l > W else 0) for l, f in enumerate(run.far_sums))


def test_split_schedule_needs_the_claims():
    """Without the chain's own claim of an untaken row (a chain that always
    waits for a helper), a run with the helpers admitted after the chain
    finishes can deadlock: the check above would catch a protocol that let
    the chain wait on a CTA that has not started."""
    W, PW = _defaults()

    class _NoClaim(_Run):
        def chain(self, rank):
            W, PW, t = self.W, self.PW, self.tb
            for l in range(rank, self.nblk, self.cs):
                helped = l > W
                acc = self.b[l * t:(l + 1) * t].copy()
                for j in range(l - W if helped else 0, l - 1):
                    yield lambda j=j: self.xflag[j]
                    acc -= self.blk(l, j) @ self.X[j * t:(j + 1) * t]
                    if helped and j == l - PW:
                        yield lambda: self.rowst[l] == 3
                        acc -= self.part[l * t:(l + 1) * t]
                y = np.linalg.solve(self.blk(l, l), acc)
                if l > 0:
                    yield lambda: self.xflag[l - 1]
                    M = np.linalg.solve(self.blk(l, l), self.blk(l, l - 1))
                    y = y - M @ self.X[(l - 1) * t:l * t]
                self.X[l * t:(l + 1) * t] = y
                self.xflag[l] = 1

    L, b = _system(40, 3, 0)
    run = _NoClaim(L, b, 40, 3, 4, W, PW, groups=3, capacity=1, seed=0)
    with pytest.raises(AssertionError, match="deadlock"):
        run.run()
