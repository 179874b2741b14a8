"""Local reassembly through the GB300 engine: the K-mer tally of listed reads
on the device (pg_kmer_tally_reads) against the oracle's tally of the same
reads, and --fix gaps,local end to end (device pileups, break candidates and
tallies; host recruitment, walk and GapFiller) against the oracle's
restatement of identifyAndFixIssues, byte for byte in FASTA, VCF and changes
(S/GenomeRegion.scala:307-414, 623-657, S/GapFiller.scala:28-402,
S/Assembler.scala:46-284)."""
import copy
import os
import tempfile

import numpy as np
import pytest

from oracle import oracle
from pilon_gb300 import _abi, reassembly, synth
from pilon_gb300.polish import Options, polish

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    from pilon_gb300.engine import Engine
    e = Engine(0)
    yield e
    e.close()


def _sorted_edges(e):
    key = np.lexsort((e["key3"], e["key2"], e["key1"], e["key0"], e["window"]))
    return e[key]


@pytest.mark.parametrize("K", [31, 47, 63])
def test_kmer_tally_reads_matches_oracle(engine, K):
    """Windows of listed reads — the flank reads of breaks with stray mates
    from elsewhere in the store, an empty list, a list out of store order —
    give the oracle's edges exactly."""
    ds = synth.generate(4, 0.01)
    params = _abi.default_params()
    engine.set_reference(ds.contigs)
    engine.set_reads(ds.reads)
    bam = reassembly.BamState(ds.reads, params, len(ds.contigs))
    rng = np.random.default_rng(K)
    lists = [bam.recruit(0, s, s + int(rng.integers(1, 400)))
             for s in rng.integers(2_000, ds.contigs[0].size - 2_000, size=16).tolist()]
    # windows that reach one read of an improper pair and not its mate: the mate is recruited as a stray
    r = ds.reads
    strays = np.nonzero(((r.flag & 0x3) == 0x1) & ((r.flag & 0x500) == 0))[0]
    flank = bam.max_insert_size()
    for i in rng.choice(strays, size=8, replace=False).tolist():
        lists.append(bam.recruit(0, int(r.pos[i]) + flank, int(r.pos[i]) + flank))
    lists.append(np.zeros(0, np.int64))
    lists.append(rng.permutation(lists[0]))
    assert any(np.any(np.diff(x) < 0) for x in lists[:-2])  # stray mates appended after the flank reads
    got = _sorted_edges(engine.kmer_tally_reads(lists, K, params))
    parts = []
    for w, lst in enumerate(lists):
        sub = ds.reads.subset(lst)
        e = oracle.kmer_tally_wide(sub, params, [(0, sub.n_reads)], K)
        e["window"] = w
        parts.append(e)
    want = _sorted_edges(np.concatenate(parts))
    assert got.size == want.size > 0
    assert np.array_equal(got, want)


def _compare(engine, ds, **kw):
    params = _abi.default_params()
    opts = Options(**kw)
    with tempfile.TemporaryDirectory() as d:
        g, o = os.path.join(d, "gpu"), os.path.join(d, "ora")
        polish(engine, ds.names, ds.contigs, ds.reads, params, g, opts)
        assert oracle.polish(ds.reads, params, ds.names, ds.contigs, o, chunk_size=opts.chunk_size,
                             fix_snps=opts.fix_snps, fix_indels=opts.fix_indels, fix_gaps=opts.fix_gaps,
                             fix_local=opts.fix_local, K=opts.K, strays=opts.strays) == 0
        out = {}
        for ext in ("fasta", "changes", "vcf"):
            a, b = open(f"{g}.{ext}", "rb").read(), open(f"{o}.{ext}", "rb").read()
            if a != b:
                la, lb = a.split(b"\n"), b.split(b"\n")
                for k, (x, y) in enumerate(zip(la, lb)):
                    if x != y:
                        raise AssertionError(f"{ext} line {k}:\n gpu    {x[:300]!r}\n oracle {y[:300]!r}")
                raise AssertionError(f"{ext}: {len(la)} vs {len(lb)} lines")
            out[ext] = a
        return out


@pytest.mark.parametrize("K", [31, 47])
def test_fix_all_eukaryotic_with_gaps(engine, K):
    """--fix all (snps, indels, gaps, local) on 6 Mb of the repeat-rich
    workload, with a closable 60 bp gap and a 3 kb gap whose middle no read
    covers."""
    ds = copy.copy(synth.generate(4, 0.05))
    ref = ds.contigs[0].copy()
    ref[1_200_000:1_200_060] = ord("N")
    ref[3_500_000:3_503_000] = ord("N")
    ds.contigs = [ref]
    r = ds.reads
    ds.reads = r.subset(np.nonzero((r.aend < 3_501_000) | (r.pos > 3_502_000))[0])
    out = _compare(engine, ds, fix_gaps=True, fix_local=True, K=K)
    big = [l for l in out["changes"].decode().splitlines()
           if max(len(l.split()[2].strip(".")), len(l.split()[3].strip("."))) > 10]
    assert len(big) >= 40
    assert out["vcf"].count(b"IMPRECISE\tGT\t1/1") >= 1  # the partial gap fill


def test_fix_all_many_contigs(engine):
    """--fix all over 30 uneven contigs of the draft workload, no strays."""
    ds = synth.generate(3, scale=0.01)
    _compare(engine, ds, fix_gaps=True, fix_local=True, K=31, strays=False)
    _compare(engine, ds, fix_gaps=True, fix_local=True, K=47)
