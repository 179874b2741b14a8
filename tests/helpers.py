"""Shared helpers of the test-suite: run the engine and the oracle on the same
regions and compare every array."""
from oracle import oracle
from pilon_gb300.regions import plan_regions

from oracle.parity import FIELDS, STATS, compare_region  # noqa: F401  (re-exported for the tests)


def oracle_regions(ds, params, regions):
    out = []
    for (c, s, e, rb, re) in regions:
        out.append(oracle.process_region(ds.reads, params, ds.contigs[c], c, s, e, rb, re))
    return out


def plan(ds, chunk_size=10_000_000, targets=None):
    return plan_regions(ds.reads, [c.size for c in ds.contigs], chunk_size, targets)
