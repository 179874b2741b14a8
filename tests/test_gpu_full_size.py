"""Full-size workloads against the oracle, every region and every field.

The other GPU tests compare scaled-down cases; these run the benchmark
workloads at their full sizes through the C ABI and compare each region's
pileup counters, calls, scores, indel strings and statistics with the oracle
(which runs on all host threads):

  bacterial-5Mb-100x        one 5 Mb region (multi-pass tiles, the region
                            edges of a real chunk), plus FASTA / VCF / changes
                            byte for byte
  draft-3000-contigs-40x    3,000 uneven contigs in one batched plan and on
                            the per-region path
  eukaryotic-120Mb-repeats  twelve 10 Mb chunks of one contig (regions that
                            start inside the contig, reads fed to two chunks),
                            the K-mer graphs of all 2,000 reassembly windows,
                            and --fix snps,indels,gaps,local --K 31 end to end
                            (FASTA and changes byte for byte)
"""
import os

import numpy as np
import pytest

from oracle import oracle
from oracle.parity import full_parity
from pilon_gb300 import _abi, synth
from tests.helpers import plan

pytestmark = pytest.mark.gpu

THREADS = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


@pytest.fixture(scope="module")
def engine():
    from pilon_gb300.engine import Engine
    e = Engine(0)
    yield e
    e.close()


def load(engine, ds):
    engine.set_reference(ds.contigs)
    engine.set_reads(ds.reads)


def test_full_bacterial_5mb(engine):
    ds = synth.generate(2)
    regions = plan(ds)
    assert len(regions) == 1 and regions[0][2] - regions[0][1] + 1 == 5_000_000
    load(engine, ds)
    n_reg, n_pos = full_parity(engine, ds, _abi.default_params(), regions, THREADS)
    assert (n_reg, n_pos) == (1, 5_000_000)
    from tests.test_gpu_outputs import compare_outputs
    compare_outputs(engine, ds)


def test_full_many_contigs_batched_and_plain(engine):
    ds = synth.generate(3)
    regions = plan(ds)
    assert len(regions) == len(ds.contigs) == 3000
    load(engine, ds)
    p = _abi.default_params()
    n_reg, n_pos = full_parity(engine, ds, p, regions, THREADS, batched=True)
    assert n_reg == 3000 and n_pos == sum(c.size for c in ds.contigs)
    n_reg, _ = full_parity(engine, ds, p, regions, THREADS, batched=False)
    assert n_reg == 3000


@pytest.fixture(scope="module")
def cfg4():
    return synth.generate(4)


def test_full_eukaryotic_chunks_and_kmer_windows(engine, cfg4):
    ds = cfg4
    regions = plan(ds)
    assert len(regions) == 12
    load(engine, ds)
    p = _abi.default_params()
    n_reg, n_pos = full_parity(engine, ds, p, regions, THREADS)
    assert (n_reg, n_pos) == (12, 120_000_000)
    # the K-mer tally (K = 31) of one window per planted indel, every window
    from pilon_gb300.regions import ReadIndex
    idx = ReadIndex(ds.reads, len(ds.contigs))
    wins = []
    for ci, var in enumerate(ds.variants):
        n = ds.contigs[ci].size
        for v in var:
            wins.append(idx.range_for(ci, max(1, v[0] - 500), min(n, v[0] + 500), n, slop=0))
    assert len(wins) == 2000
    got = engine.kmer_tally(wins, 31, p)
    import threading
    parts = [list(range(k, len(wins), THREADS)) for k in range(THREADS)]
    res = [None] * THREADS

    def worker(k):
        if parts[k]:
            res[k] = oracle.kmer_tally(ds.reads, p, [wins[w] for w in parts[k]], 31)
    ths = [threading.Thread(target=worker, args=(k,)) for k in range(THREADS)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    cols = ["key_hi", "key_lo", "next", "alt", "depth", "weight"]

    def rows(e, wmap):
        a = np.stack([wmap(e["window"].astype(np.int64))] + [e[c].astype(np.int64) for c in cols], axis=1)
        return a[np.lexsort(a.T[::-1])]
    want = np.concatenate([rows(res[k], lambda w, k=k: np.array(parts[k], np.int64)[w])
                           for k in range(THREADS) if res[k] is not None])
    want = want[np.lexsort(want.T[::-1])]
    have = rows(got, lambda w: w)
    assert have.shape == want.shape, (have.shape, want.shape)
    assert np.array_equal(have, want)


def test_full_eukaryotic_fix_all(engine, cfg4):
    """Pilon's default --fix (snps, indels, gaps, local) with --K 31 over the
    whole 120 Mb workload: device pileups, breaks and K-mer tallies, host
    recruitment and graph walks, against the oracle's restatement of
    processRegions with GapFiller (on all host threads).  The FASTA and the
    changes are compared byte for byte; the VCF, about 18 GB at this size, is
    compared on 6 Mb of the workload in tests/test_gpu_reassembly.py."""
    import tempfile
    from pilon_gb300.polish import Options, polish
    ds = cfg4
    p = _abi.default_params()
    stats = {}
    with tempfile.TemporaryDirectory() as d:
        g, o = os.path.join(d, "gpu"), os.path.join(d, "ora")
        polish(engine, ds.names, ds.contigs, ds.reads, p, g, Options(vcf=False, fix_gaps=True, fix_local=True, K=31))
        assert oracle.polish(ds.reads, p, ds.names, ds.contigs, o, fix_gaps=True, fix_local=True, K=31, vcf=False,
                             stats=stats) == 0
        for ext in ("changes", "fasta"):
            a, b = open(f"{g}.{ext}", "rb").read(), open(f"{o}.{ext}", "rb").read()
            assert a == b, ext
        lines = open(f"{g}.changes").read().splitlines()
    big = [l for l in lines if max(len(l.split()[2].strip(".")), len(l.split()[3].strip("."))) > 10]
    assert len(big) >= 1000, len(big)
    assert stats["tied_sets"] == 0  # no join set where the Scala HashSet's order would decide
