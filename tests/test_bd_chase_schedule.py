"""The band chase's concurrent schedule gives the sequential result.

DDLA's Bd2Bi (DDLA/Transformations/Bidiagonaling.cs:478-516) runs the
bulge-chasing cycles one after another.  The GPU kernel (bidiag2s.cu,
k_bd_chase) runs consecutive cycles on different CTAs: cycle s starts its
t-th reflector once cycle s - 1 has finished min(t + LAG, all) of its own.
Every reflector reads and writes one rectangle of the band (its StepSide
view), so the concurrent run equals the sequential one when every pair of
reflectors that the rule lets run at the same time, or in the other order,
touches disjoint rectangles.  This test enumerates those pairs for many
sizes, with LAG and the block width read from the kernel source, and checks
that a smaller LAG would not be safe (so the check sees overlaps).
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "ddla_gb300", "csrc", "bidiag2s.cu")


def _const(name):
    m = re.search(r"constexpr int " + name + r"\s*=\s*(\d+);", open(SRC).read())
    assert m, name
    return int(m.group(1))


def cycle_rects(n, s, bs):
    """The rectangles (r0, r1, c0, c1) of W that cycle s's reflectors touch,
    in order (Bd2Bi_StepCycle, Bidiagonaling.cs:489-516)."""
    rows = n - s
    out = []

    def side(r0, nr, c0, nc):
        out.append((s + r0, s + r0 + nr, s + c0, s + c0 + nc))

    is_, ie = 1, 1 + bs
    if rows <= ie:
        side(0, rows, is_, rows - is_)
        side(is_, rows - is_, is_, rows - is_)
        return out
    ie2 = ie + bs
    side(0, ie, is_, ie - is_)
    while ie2 < rows:
        side(is_, ie - is_, is_, ie2 - is_)
        side(is_, ie2 - is_, ie, ie2 - ie)
        is_ += bs
        ie += bs
        ie2 += bs
    side(is_, ie - is_, is_, rows - is_)
    side(is_, rows - is_, ie, rows - ie)
    side(ie, rows - ie, ie, rows - ie)
    return out


def _overlap(a, b):
    return a[0] < b[1] and b[0] < a[1] and a[2] < b[3] and b[2] < a[3]


def schedule_conflicts(n, lag):
    bs = min(n, _const("BD2_BLOCK"))
    cyc = [cycle_rects(n, s, bs) for s in range(n - 1)]
    bad = []
    for s in range(1, n - 1):
        for t, rect in enumerate(cyc[s]):
            # steps of cycle s - k at index >= g are not known to be finished
            # when (s, t) runs: they may run at the same time or later
            g = min(t + lag, len(cyc[s - 1]))
            k = 1
            while s - k >= 0 and g < len(cyc[s - k]):
                for t2 in range(g, len(cyc[s - k])):
                    if _overlap(rect, cyc[s - k][t2]):
                        bad.append((s, t, s - k, t2))
                if s - k - 1 < 0:
                    break
                # (s-k) finished g steps: its step g - 1 waited for (s-k-1)
                g = min(g - 1 + lag, len(cyc[s - k - 1]))
                k += 1
    return bad


SIZES = list(range(2, 90)) + [96, 97, 128, 129, 130, 160, 161, 193, 257]


def test_kernel_steps_match_cycle_length():
    # cycle_steps() in the kernel: 2 reflectors for a short cycle, else 2 k + 4
    src = open(SRC).read()
    assert "return 2 * k + 4;" in src and "if (rows <= 1 + bs) return 2;" in src
    for n in (5, 40, 100, 257):
        bs = min(n, _const("BD2_BLOCK"))
        for s in range(n - 1):
            rows = n - s
            k = 0
            ie2 = 1 + 2 * bs
            while ie2 < rows:
                k += 1
                ie2 += bs
            want = 2 if rows <= 1 + bs else 2 * k + 4
            assert len(cycle_rects(n, s, bs)) == want


def test_lag_in_kernel_is_safe():
    lag = _const("BD2_LAG")
    for n in SIZES:
        bad = schedule_conflicts(n, lag)
        assert not bad, f"n={n}: concurrent reflectors overlap, e.g. {bad[:3]}"


def test_smaller_lag_overlaps():
    lag = _const("BD2_LAG")
    assert any(schedule_conflicts(n, lag - 1) for n in SIZES)
