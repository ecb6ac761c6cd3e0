"""CPU: the pipeline schedule of the Ozaki GEMM kernel (k_oz_gemm), read from
its source constants and replayed on the host.

The kernel's correctness rests on three properties of its constants:
  * exactness: level l's FP32 TMEM sum over one flush period stays below 2^24
    ulps, (l + 1) * period * OZ_KC * 127^2 < 2^24;
  * at most one flush period ends on any K chunk, so the two spare TMEM slots
    (handed over in FIFO order) are always free when taken;
  * the mbarrier rings (stages, MMA-ready and flush-done rings of OZ_RING
    slots, issuer slack) never let a wait see an aliased phase parity, and no
    TMEM slot is overwritten before its flush.
The replay runs the issuer, the 8 flusher warps, the copy engine and the
in-order tensor pipe as independent agents in random interleavings.
"""
import os
import random
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "ddla_gb300", "csrc", "tcgemm.cu")


def _constants():
    s = open(SRC).read()

    def one(pat):
        m = re.search(pat, s)
        assert m, pat
        return int(m.group(1))

    def table(fn):
        body = re.search(fn + r"\(int a\) \{\s*return ([^;]*);", s).group(1)
        vals = [int(v) for v in re.findall(r"\? (\d+)", body)] + [int(re.search(r": (\d+)\s*$", body).group(1))]
        return vals

    c = {
        "KC": one(r"constexpr int OZ_KC = (\d+);"),
        "NS": one(r"constexpr int OZ_NS = (\d+);"),
        "EXACT": one(r"constexpr int OZ_EXACT = (\d+);"),
        "RING": one(r"constexpr int OZ_RING = (\d+);"),
        "SLACK": one(r"fdone\[\(c - (\d+)\) % OZ_RING\]"),
        "P": table("oz_period"),
        "O": table("oz_phase"),
    }
    assert re.search(r"constexpr int OZ_SLOTS = OZ_NACC \+ 2;", s)
    return c


def test_exact_periods_and_one_flush_per_chunk():
    c = _constants()
    P, O, KC = c["P"], c["O"], c["KC"]
    assert len(P) == len(O) == c["EXACT"] + 1
    for a in range(c["EXACT"]):
        assert (a + 1) * P[a] * KC * 127 * 127 < 2 ** 24
    assert all(0 <= o < p for o, p in zip(O, P))
    period = 1
    for p in P:
        period = period * p // __import__("math").gcd(period, p)
    for ch in range(1, 2 * period + 1):
        ends = [a for a in range(len(P)) if (ch + O[a]) % P[a] == 0]
        assert len(ends) <= 1, (ch, ends)


class _Bar:
    """mbarrier: phase count n; a wait for completion k uses parity k & 1."""

    def __init__(self, count):
        self.n, self.count, self.pend = 0, count, 0

    def arrive(self):
        self.pend += 1
        if self.pend == self.count:
            self.pend, self.n = 0, self.n + 1

    def done(self, k):
        assert self.n in (k, k + 1) or self.n < k, ("aliased phase", self.n, k)
        assert not (self.n < k and (self.n & 1) != (k & 1)), ("spurious completion", self.n, k)
        return self.n == k + 1


class _Slots:
    def __init__(self, nacc):
        self.slot, self.spare = list(range(nacc)), [nacc, nacc + 1]

    def turn(self, a):
        old = self.slot[a]
        self.slot[a] = self.spare.pop(0)
        self.spare.append(old)
        return old


def _replay(c, K, seed, warps=8):
    P, O, NS, RING, D = c["P"], c["O"], c["NS"], c["RING"], c["SLACK"]
    nacc = len(P)
    rnd = random.Random(seed)
    full = [_Bar(1) for _ in range(NS)]
    mdone = [_Bar(1) for _ in range(NS)]
    mready = [_Bar(1) for _ in range(RING)]
    fdone = [_Bar(warps) for _ in range(RING)]
    copies = [(st, st) for st in range(min(NS, K))]
    stage_of = {st: st for st in range(min(NS, K))}
    mma = []
    iss = {"c": 0, "ph": "full", "slots": _Slots(nacc)}
    fl = [{"f": 0, "slots": _Slots(nacc)} for _ in range(warps)]
    tmem = {}   # slot -> [accumulator, period index, readers, flushed]
    for _ in range(100000):
        acts = (["copy"] if copies else []) + (["mma"] if mma else []) + (["iss"] if iss["c"] < K else [])
        acts += [w for w in range(warps) if fl[w]["f"] < K]
        if not acts:
            break
        act = rnd.choice(acts)
        if act == "copy":
            st, _ch = copies.pop(0)
            full[st].arrive()
        elif act == "mma":
            ch, st, writes = mma.pop(0)
            for a, sl, fresh, ep in writes:
                if fresh:
                    old = tmem.get(sl)
                    assert old is None or old[3], ("slot overwritten before its flush", sl, old)
                    tmem[sl] = [a, ep, set(), False]
                else:
                    assert tmem[sl][:2] == [a, ep] and not tmem[sl][3]
            mdone[st].arrive()
            mready[ch % RING].arrive()
        elif act == "iss":
            ch, st = iss["c"], iss["c"] % NS
            if iss["ph"] == "full":
                assert stage_of.get(st) == ch
                if full[st].done(ch // NS):
                    iss["ph"] = "fdone"
            elif iss["ph"] == "fdone":
                if ch < D or fdone[(ch - D) % RING].done((ch - D) // RING):
                    writes = []
                    for a in range(nacc):
                        fresh = ch == 0
                        if ch > 0 and (ch + O[a]) % P[a] == 0:
                            iss["slots"].turn(a)
                            fresh = True
                        writes.append((a, iss["slots"].slot[a], fresh, (ch + O[a]) // P[a]))
                    mma.append((ch, st, writes))
                    if ch >= 1:
                        iss["ph"] = "mdone"
                    else:
                        iss["c"], iss["ph"] = ch + 1, "full"
            else:
                sp = (ch - 1) % NS
                if mdone[sp].done((ch - 1) // NS):
                    if ch - 1 + NS < K:
                        copies.append((sp, ch - 1 + NS))
                        stage_of[sp] = ch - 1 + NS
                    iss["c"], iss["ph"] = ch + 1, "full"
        else:
            w = fl[act]
            f = w["f"]
            if mready[f % RING].done(f // RING):
                if f + 1 < K:
                    reads = [(a, w["slots"].turn(a)) for a in range(nacc) if (f + 1 + O[a]) % P[a] == 0]
                else:
                    reads = [(a, w["slots"].slot[a]) for a in range(nacc)]
                for a, sl in reads:
                    d = tmem[sl]
                    assert d[0] == a and d[1] == (f + O[a]) // P[a], ("flush of the wrong period", a, f, d)
                    d[2].add(act)
                    d[3] = len(d[2]) == warps
                if f + 1 < K:
                    fdone[f % RING].arrive()
                w["f"] = f + 1
    else:
        raise AssertionError("replay did not finish")
    assert all(v[3] for v in tmem.values())


def test_pipeline_replay():
    c = _constants()
    assert c["RING"] >= c["SLACK"]
    for K in (1, 2, 3, 5, 9, 33, 70):
        for seed in range(12):
            _replay(c, K, seed)


def test_replay_detects_planted_faults():
    # the checker itself: phases that end two periods on one chunk overwrite
    # a slot before its flush; an issuer without slack waits on its own chunk
    import pytest
    c = _constants()
    bad = dict(c, O=[0] * len(c["P"]))
    with pytest.raises(AssertionError):
        for seed in range(12):
            _replay(bad, 70, seed)
    with pytest.raises(AssertionError):
        _replay(dict(c, SLACK=0), 33, 0)
