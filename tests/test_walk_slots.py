"""CPU restatements of the pileup walk's index arithmetic, each tied to the
kernel's source lines.

Slot assignment (k_walk, the rounds of walk entries): each lane holding an
entry (one M/=/X or S operator of a read) computes its entry's slot in the
warp's round order from ballots and population counts.  The slots must be a
permutation of 0 .. n_active - 1 (every entry walked exactly once), and with 4
or 8 lane groups the first 4 * m slots of the entries of the most common mq
must hold one entry of each position residue class in every group of four
(their shared-memory atomics then fall in different banks).

Read ranges (k_tile_ranges): the warp's 32-ary lower bound over a tile's
position-sorted reads must equal a binary search, with every load in range.

Flush (k_walk): the packed per-position counters must give PileUp.add's sums
exactly for any most common mq and up to 4095 reads per pass."""
import random

import pytest


def popc(x):
    return bin(x).count("1")


def assign(sm_all, set_a, cls, ng):
    """slot per lane, as the kernel computes it (one lane at a time here)."""
    def ballot(mask, pred):
        return sum(1 << ln for ln in range(32) if mask >> ln & 1 and pred(ln))

    c = [ballot(set_a, lambda ln, k=k: cls[ln] == k) for k in range(4)]
    m = min(popc(x) for x in c)
    rank = {ln: popc(c[cls[ln]] & ((1 << ln) - 1)) for ln in range(32) if set_a >> ln & 1}
    left = ballot(set_a, lambda ln: rank[ln] >= m)
    slots = {}
    for ln in range(32):
        if not sm_all >> ln & 1:
            continue
        below = (1 << ln) - 1
        if set_a >> ln & 1:
            if ng in (4, 8):
                r = rank[ln]
                slots[ln] = 4 * r + cls[ln] if r < m else 4 * m + popc(left & below)
            else:
                slots[ln] = popc(set_a & below)
        else:
            slots[ln] = popc(set_a) + popc(sm_all & ~set_a & below)
    return slots, m


def check(sm_all, set_a, cls, ng):
    slots, m = assign(sm_all, set_a, cls, ng)
    assert sorted(slots.values()) == list(range(popc(sm_all))), (hex(sm_all), hex(set_a))
    if ng in (4, 8):
        by_slot = {s: ln for ln, s in slots.items()}
        for k in range(m):
            assert sorted(cls[by_slot[4 * k + j]] for j in range(4)) == [0, 1, 2, 3]


@pytest.mark.parametrize("ng", [2, 4, 8])
def test_random_lane_sets(ng):
    rng = random.Random(ng)
    for _ in range(3000):
        sm_all = rng.getrandbits(32) & rng.getrandbits(32) if rng.random() < 0.5 else rng.getrandbits(32)
        set_a = sm_all & (rng.getrandbits(32) if rng.random() < 0.7 else 0xFFFFFFFF)
        cls = [rng.randrange(4) if rng.random() < 0.8 else 0 for _ in range(32)]
        check(sm_all, set_a, cls, ng)


@pytest.mark.parametrize("ng", [4, 8])
def test_edge_lane_sets(ng):
    full = 0xFFFFFFFF
    for sm_all, set_a in [(0, 0), (1, 1), (full, full), (full, 0), (full, 0x0000FFFF), (0x80000000, 0x80000000)]:
        for cls in ([0] * 32, [ln % 4 for ln in range(32)], [3 - ln % 4 for ln in range(32)],
                    [ln // 8 for ln in range(32)]):
            check(sm_all, set_a, cls, ng)


def test_kernel_still_uses_these_formulas():
    """The restatement above follows these lines of the walk kernel; a change
    there must be carried over here."""
    import os
    src = open(os.path.join(os.path.dirname(__file__), "..", "pilon_gb300", "csrc", "pg_pileup.cu")).read()
    for line in ["slot = rank < m ? 4 * rank + cls : 4 * m + __popc(left & below);",
                 "slot = __popc(set_a & below);",
                 "slot = __popc(set_a) + __popc(act_all & ~set_a & below);"]:
        assert line in src, line


def warp_lower_bound(pos, lo, hi, v):
    """k_tile_ranges' warp_lower_bound_pos: 32 lanes sample [lo, hi) at even
    strides per step; every load stays below hi."""
    while hi - lo > 32:
        step = (hi - lo + 31) // 32
        below = 0
        for lane in range(32):
            sk = lo + lane * step
            if sk < hi and pos[sk] < v:
                below |= 1 << lane
        c = popc(below)
        if c == 0:
            return lo
        nlo = lo + (c - 1) * step + 1
        sc = lo + c * step
        hi = sc if (c < 32 and sc < hi) else hi
        lo = nlo
    return lo + sum(1 for lane in range(32) if lo + lane < hi and pos[lo + lane] < v)


def test_warp_lower_bound_matches_bisect():
    """The first index of [lo, hi) whose position is >= v, for sorted positions
    with many duplicates, empty and short ranges, and v outside the values."""
    import bisect
    rng = random.Random(9)
    for _ in range(2500):
        n = rng.choice([0, 1, 5, 31, 32, 33, 64, 100, 1000, 5000])
        pos = sorted(rng.randrange(0, max(1, n // rng.choice([1, 3, 50]))) for _ in range(n))
        lo = rng.randrange(0, n + 1)
        hi = rng.randrange(lo, n + 1)
        v = rng.randrange(-2, (pos[-1] + 3) if pos else 3)
        assert warp_lower_bound(pos, lo, hi, v) == bisect.bisect_left(pos, v, lo, hi), (n, lo, hi, v)


def test_kernel_lower_bound_lines():
    import os
    src = open(os.path.join(os.path.dirname(__file__), "..", "pilon_gb300", "csrc", "pg_pileup.cu")).read()
    for line in ["const int64_t step = (hi - lo + 31) / 32;",
                 "const unsigned below = __ballot_sync(FULL, sk < hi && (int64_t)pos[sk] < v);",
                 "const int64_t nlo = lo + (int64_t)(c - 1) * step + 1;",
                 "hi = (c < 32 && sc < hi) ? sc : hi;",
                 "const unsigned below = __ballot_sync(FULL, lo + lane < hi && (int64_t)pos[lo + lane] < v);"]:
        assert line in src, line


def _flush(reads, M):
    """One position of one walk pass: the packed shared-memory words as the walk
    adds to them (md[b] += qual + (1 << 20); for mq + 1 != M also qx[b] +=
    qual * (mq + 1 - M) and mx += mq + 1 - M, all uint32) and the flush that
    turns them into qualSum, mqSum, qSum and the counts."""
    U = 0xFFFFFFFF
    md, qx, mx = [0] * 4, [0] * 4, 0
    for b, q, mq1 in reads:
        md[b] = (md[b] + q + (1 << 20)) & U
        d = mq1 - M
        if d:
            qx[b] = (qx[b] + q * d) & U
            mx = (mx + d) & U
    s32 = lambda x: x - (1 << 32) if x >= 1 << 31 else x
    counts = [w >> 20 for w in md]
    sums = [w & 0xFFFFF for w in md]
    qual_sum = [M * sums[b] + s32(qx[b]) for b in range(4)]
    mq_sum = s32((M * sum(counts) + mx) & U)
    return counts, qual_sum, mq_sum, sum(sums)


@pytest.mark.parametrize("case", ["max_up", "max_down", "random"])
def test_walk_flush_is_exact_up_to_4095_reads(case):
    """PileUp.add sums (count, qualSum as Long, mqSum, qSum) from the packed
    counters, exact for any most common mq + 1 = M and up to 4095 reads per pass
    (qualities are bytes, at most 127): 4095 reads at quality 127 and mq + 1 = 256
    with M = 1, the reverse, and random mixes."""
    rng = random.Random(17)
    trials = 1 if case != "random" else 300
    for _ in range(trials):
        if case == "max_up":
            M, reads = 1, [(rng.randrange(4), 127, 256) for _ in range(4095)]
        elif case == "max_down":
            M, reads = 256, [(rng.randrange(4), 127, 1) for _ in range(4095)]
        else:
            M = rng.randrange(1, 257)
            reads = [(rng.randrange(4), rng.randrange(128), rng.randrange(1, 257))
                     for _ in range(rng.randrange(0, 4096))]
        counts, qual_sum, mq_sum, q_sum = _flush(reads, M)
        assert counts == [sum(1 for b, _, _ in reads if b == k) for k in range(4)]
        assert qual_sum == [sum(q * m for b, q, m in reads if b == k) for k in range(4)]
        assert mq_sum == sum(m for _, _, m in reads) and q_sum == sum(q for _, q, _ in reads)


def test_kernel_flush_lines():
    import os
    csrc = os.path.join(os.path.dirname(__file__), "..", "pilon_gb300", "csrc")
    src = open(os.path.join(csrc, "pg_pileup.cu")).read() + open(os.path.join(csrc, "pg_internal.cuh")).read()
    for line in ["const uint32_t s0 = w0 & 0xFFFFFu, s1 = w1 & 0xFFFFFu, s2 = w2 & 0xFFFFFu, s3 = w3 & 0xFFFFFu;",
                 "const longlong2 q01 = make_longlong2((long long)M * s0 + (int32_t)sm[4 * T + p],",
                 "const int32_t mqs = wadd((int32_t)(M * (uint32_t)(c.x + c.y + c.z + c.w)), (int32_t)sm[8 * T + p]);",
                 "atomicAdd(c, (uint32_t)qual + (1u << 20));",
                 "atomicAdd(c + 4 * T, (uint32_t)(qual * dmq));",
                 "atomicAdd(sm + 8 * T + p, (uint32_t)dmq);",
                 "constexpr int64_t kMaxReadsPerPass = 4095;"]:
        assert line in src, line
