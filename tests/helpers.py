"""Shared helpers of the test-suite: run the engine and the oracle on the same
regions and compare every array."""
import numpy as np

from oracle import oracle
from pilon_gb300 import _abi
from pilon_gb300.regions import plan_regions

FIELDS = ["count", "qual_sum", "mq_sum", "q_sum", "phys_cov", "insert_size", "bad_pair", "deletions", "del_qual",
          "insertions", "ins_qual", "clips", "call", "score", "indel_len"]
STATS = ["base_count", "read_count", "phys_cov_start", "insert_size_start", "min_depth", "n_changes", "fr_count",
         "fr_sum", "fr_sumsq", "rf_count", "rf_sum", "rf_sumsq", "error"]


def oracle_regions(ds, params, regions):
    out = []
    for (c, s, e, rb, re) in regions:
        out.append(oracle.process_region(ds.reads, params, ds.contigs[c], c, s, e, rb, re))
    return out


def compare_region(gpu, ora, label=""):
    """Asserts bit-exact equality of every field; returns the number of positions."""
    for f in FIELDS:
        a, b = getattr(gpu, f), getattr(ora, f)
        if not np.array_equal(a, b):
            bad = np.nonzero(a != b)[0]
            i = int(bad[0])
            pos = i // 4 if f in ("count", "qual_sum") else i
            raise AssertionError(f"{label} field {f}: {bad.size} mismatches, first at index {i} (position {pos}):"
                                 f" gpu={a[i]} oracle={b[i]}")
    for i in np.nonzero(gpu.call & _abi.PG_CALL_INS)[0][:2000]:
        assert gpu.insertion(i) == ora.insertion(i), f"{label} insertion string at {i}"
    for f in STATS:
        assert getattr(gpu.stats, f) == getattr(ora.stats, f), f"{label} stat {f}: {getattr(gpu.stats, f)} != " \
                                                              f"{getattr(ora.stats, f)}"
    return gpu.size


def plan(ds, chunk_size=10_000_000, targets=None):
    return plan_regions(ds.reads, [c.size for c in ds.contigs], chunk_size, targets)
