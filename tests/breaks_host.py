"""Test support: break candidates of a region (GenomeRegion.possibleBreaks,
S/GenomeRegion.scala:659-763 and pctBadOverall :99-114), computed on the host
from the engine's per-position arrays, to check the device's pg_find_breaks.  These regions are the windows whose reads the
K-mer tally consumes (S/GenomeRegion.scala:395-410)."""
import numpy as np


def smooth(inp, window):
    """GenomeRegion.smooth (S/GenomeRegion.scala:190-210), same integer steps."""
    n = inp.size
    res = np.zeros(n, np.int64)
    half = window // 2
    if n > window:
        cs = np.concatenate([[0], np.cumsum(inp.astype(np.int64))])
        i = np.arange(window + 1, n)
        # after step i the accumulator holds input[0] + input[i-window+1 .. i]
        acc = inp[0] + (cs[i + 1] - cs[i - window + 1])
        res[i - half] = (acc + half) // window
        res[:window - half] = res[window - half]
        res[n - half:] = res[n - half - 1]
    else:
        res[:] = int(inp.astype(np.int64).sum()) // n
    return res


def java_round(x):
    f = np.floor(x)
    return np.where(x - f >= 0.5, f + 1, f).astype(np.int64)


def summary_regions(test, start, stop, slop):
    """GenomeRegion.summaryRegions (S/GenomeRegion.scala:743-763) on a boolean array.
    A run closes at the first untested position more than `slop` past its last
    tested one, so tested positions up to slop + 1 apart share a run."""
    idx = np.nonzero(test)[0]
    regs = []
    if idx.size:
        gaps = np.nonzero(np.diff(idx) > slop + 1)[0]
        firsts = np.concatenate([[idx[0]], idx[gaps + 1]])
        lasts = np.concatenate([idx[gaps], [idx[-1]]])
        regs = [(start + int(a), start + int(b)) for a, b in zip(firsts, lasts)]
    return [r for r in regs if not (r[0] - start < 100 or stop - r[1] < 100)]



def _pct_int(n, d):
    """Utils.pct(Int, Int) = roundDiv(100 * n, d) with 32-bit wrap-around."""
    n100 = (100 * n.astype(np.int64) + 2**31) % 2**32 - 2**31
    num = (n100 + d // 2 + 2**31) % 2**32 - 2**31
    with np.errstate(divide="ignore", invalid="ignore"):
        q = np.where(d > 0, np.trunc(num / np.where(d > 0, d, 1)), 0)
    return q.astype(np.int64)


def region_arrays(counts, deletions, bad_pair, clips, call, indel_len, read_count):
    """coverage, badCoverage, clips (pass 1, S/GenomeRegion.scala:247-253) and
    fragCoverage (processBam, :287-300) from the fetched pileups."""
    n = deletions.size
    depth = counts.reshape(-1, 4).astype(np.int64).sum(1) + deletions
    frag = depth.copy()
    kind = (call >> 9) & 7
    for i in np.nonzero(kind == 3)[0].tolist():  # undo the deletion-span update for fragCoverage
        frag[i + 1:i + int(indel_len[i])] -= int(deletions[i])
    if read_count == 0:  # postProcess returns before pass 1
        z = np.zeros(n, np.int64)
        return z, z, z, frag
    cl = clips.astype(np.int16).astype(np.int64)  # pu.clips.toShort
    return depth, bad_pair.astype(np.int64), cl, frag


def possible_breaks(coverage, bad, clips, frag, ref_region, start, stop, min_min_depth=5):
    size = coverage.size
    refu = np.frombuffer(bytes(ref_region).upper(), np.uint8)
    isN = refu == ord("N")
    mean = float(frag.sum()) / size
    tot_bad, tot_good = int(bad.sum()), int(coverage.sum())
    d = tot_good + tot_bad
    pbo = (100 * tot_bad + d // 2) // d if d > 0 else 0
    low = (coverage < min_min_depth) & ~isN
    high = (coverage >= min_min_depth) & (_pct_int(clips, coverage) >= 33)
    too_bad = _pct_int(bad, coverage + bad) > pbo + 20
    idx = np.arange(size)
    left = frag[np.maximum(0, idx - 100)]
    right = frag[np.minimum(size - 1, idx + 100)]
    dip = (left - frag) + (right - frag)
    with np.errstate(divide="ignore", invalid="ignore"):
        dipf = dip / mean if mean != 0 else np.where(dip > 0, np.inf, np.where(dip < 0, -np.inf, np.nan))
        dipb = dipf >= 1.5
    brk = low | high | too_bad | dipb
    regs = summary_regions(brk, start, stop, 200)
    gaps = [g for g in summary_regions(isN, start, stop, 100) if g[1] + 1 - g[0] >= 10]

    def near(r):  # Region.near with distance 300 (S/Region.scala:41-44)
        for g in gaps:
            if (g[0] <= r[1] and g[1] >= r[0]) or abs(g[1] - r[0]) <= 300 or abs(g[0] - r[1]) <= 300:
                return True
        return False
    return [r for r in regs if not near(r)]
