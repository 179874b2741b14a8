"""Region-by-region comparison of the engine's results with the oracle's.

TEST INFRASTRUCTURE ONLY: used by tests/ and by bench.py's CPU
baseline leg, never by the pilon_gb300 product path.  Every pileup counter,
call flag, score, indel length and string and region statistic must be equal
bit for bit.
"""
import queue
import threading

import numpy as np

from pilon_gb300 import _abi

from . import oracle

FIELDS = ["count", "qual_sum", "mq_sum", "q_sum", "phys_cov", "insert_size", "bad_pair", "deletions", "del_qual",
          "insertions", "ins_qual", "clips", "call", "score", "indel_len"]
STATS = ["base_count", "read_count", "phys_cov_start", "insert_size_start", "min_depth", "n_changes", "fr_count",
         "fr_sum", "fr_sumsq", "rf_count", "rf_sum", "rf_sumsq", "error"]


def compare_region(gpu, ora, label="", max_strings=None):
    """Asserts bit-exact equality of every field; returns the number of positions."""
    for f in FIELDS:
        a, b = getattr(gpu, f), getattr(ora, f)
        if not np.array_equal(a, b):
            bad = np.nonzero(a != b)[0]
            i = int(bad[0])
            pos = i // 4 if f in ("count", "qual_sum") else i
            raise AssertionError(f"{label} field {f}: {bad.size} mismatches, first at index {i} (position {pos}):"
                                 f" gpu={a[i]} oracle={b[i]}")
    ins = np.nonzero(gpu.call & _abi.PG_CALL_INS)[0]
    if max_strings is not None:
        ins = ins[:max_strings]
    for i in ins:
        assert gpu.insertion(i) == ora.insertion(i), f"{label} insertion string at {i}"
    for f in STATS:
        assert getattr(gpu.stats, f) == getattr(ora.stats, f), f"{label} stat {f}: {getattr(gpu.stats, f)} != " \
                                                              f"{getattr(ora.stats, f)}"
    return gpu.size


def full_parity(engine, ds, params, regions, threads, batched=True):
    """Runs the engine once over all regions, then the oracle on every region on
    `threads` host threads (largest regions first), comparing each region as
    its oracle result arrives.  At most `threads` oracle results are held at
    once, so the host memory stays bounded at full size.  Returns
    (regions compared, positions compared); raises AssertionError on the first
    difference."""
    engine.pileup_regions(regions, params, batched=batched)
    order = sorted(range(len(regions)), key=lambda r: regions[r][1] - regions[r][2])
    it = iter(order)
    lock = threading.Lock()
    done = queue.Queue(maxsize=max(1, threads))
    stop = threading.Event()

    def worker():
        while not stop.is_set():
            with lock:
                r = next(it, None)
            if r is None:
                done.put(None)
                return
            c, s, e, rb, re = regions[r]
            try:
                res = oracle.process_region(ds.reads, params, ds.contigs[c], c, s, e, rb, re)
            except Exception as ex:  # noqa: BLE001  (re-raised on the main thread)
                res = ex
            done.put((r, res))

    ths = [threading.Thread(target=worker, daemon=True) for _ in range(threads)]
    for t in ths:
        t.start()
    finished, n_reg, n_pos = 0, 0, 0
    try:
        while finished < threads:
            item = done.get()
            if item is None:
                finished += 1
                continue
            r, ora = item
            if isinstance(ora, Exception):
                raise ora
            n_pos += compare_region(engine.fetch(r), ora, label=f"region {r} {regions[r][:3]}")
            n_reg += 1
    finally:
        stop.set()
        while any(t.is_alive() for t in ths):  # let the workers leave
            try:
                done.get(timeout=0.1)
            except queue.Empty:
                pass
    return n_reg, n_pos
