"""Sharding regions over several GPUs (one process per GPU).

Regions are independent (S/GenomeFile.scala:101-120 processes them one after
another with no shared state except BamFile's cumulative insert statistics),
so N ranks each take a contiguous, size-balanced slice of the region list; no
collective runs on the data path.  Rank outputs are concatenated in region
order, and the insert-statistics deltas of every region are folded in region
order on the host, which reproduces the reference's running totals
(S/BamFile.scala:137, 156-202).
"""


def shard_regions(regions, world):
    """Contiguous slices of `regions` (list of (contig, start, stop, ...)) with
    about equal numbers of positions; returns a list of index lists."""
    sizes = [r[2] - r[1] + 1 for r in regions]
    total = sum(sizes)
    out = [[] for _ in range(world)]
    acc = 0
    for i, s in enumerate(sizes):
        k = min(world - 1, (acc + s // 2) * world // max(total, 1))
        out[k].append(i)
        acc += s
    return out


def fold_insert_stats(stats):
    """Running FR/RF insert statistics after each region, in region order:
    [(fr_count, fr_sum, fr_sumsq, rf_count, rf_sum, rf_sumsq)]."""
    run = [0] * 6
    out = []
    for s in stats:
        for k, f in enumerate(("fr_count", "fr_sum", "fr_sumsq", "rf_count", "rf_sum", "rf_sumsq")):
            run[k] += int(getattr(s, f) if not isinstance(s, dict) else s[f])
        out.append(tuple(run))
    return out
