"""Synthetic workloads and region planning (host logic, CPU only)."""
import numpy as np
import pytest

from pilon_gb300 import synth
from pilon_gb300.reads import CIGAR_OPS, build_store, concat_stores
from pilon_gb300.regions import contig_regions, parse_targets, plan_regions


def test_generator_is_deterministic():
    a = synth.generate(1, scale=0.2)
    b = synth.generate(1, scale=0.2)
    for f in ("pos", "aend", "flag", "mapq", "tlen", "cigar", "seq", "qual"):
        assert np.array_equal(getattr(a.reads, f), getattr(b.reads, f)), f
    assert all(np.array_equal(x, y) for x, y in zip(a.contigs, b.contigs))


def test_reads_are_consistent():
    d = synth.generate(2, scale=0.01)
    r = d.reads
    assert np.all(np.diff(r.pos) >= 0)
    for i in range(0, r.n_reads, 97):
        ops = r.read_cigar(i)
        ref_len = sum(n for n, op in ops if op in "MDN=X")
        read_len = sum(n for n, op in ops if op in "MIS=X")
        assert r.aend[i] == r.pos[i] + ref_len - 1
        assert read_len == r.l_seq[i]
    # mapq-0 fraction and flags present
    assert 0.01 < np.mean(r.mapq == 0) < 0.06
    assert np.any(r.flag & 0x400) and np.any(r.flag & 0x100)


def test_variants_present_in_reads():
    d = synth.generate(1)
    kinds = {v[1] for v in d.variants[0]}
    assert kinds == {"snp", "ins", "del"}
    r = d.reads
    ops = r.cigar & 15
    assert np.any(ops == CIGAR_OPS.index("I")) and np.any(ops == CIGAR_OPS.index("D"))
    assert np.any(ops == CIGAR_OPS.index("S"))


def test_region_read_ranges_cover_the_query_window():
    d = synth.generate(3, scale=0.005)
    lens = [c.size for c in d.contigs]
    regs = plan_regions(d.reads, lens, chunk_size=5000)
    r = d.reads
    for (c, s, e, a, b) in regs:
        qs, qe = max(s - 10000, 0), min(e + 10000, lens[c])
        sel = (r.ref_id == c) & (r.pos <= qe) & (r.aend >= qs)
        idx = np.nonzero(sel)[0]
        assert idx.size == 0 or (idx.min() >= a and idx.max() < b)


def test_targets():
    names, lens = ["a", "b"], [1000, 500]
    assert parse_targets("a:10-20,b", names, lens) == [(0, 10, 20), (1, 1, 500)]


def test_targets_file(tmp_path):
    """parseTargets reads a file of target strings first (S/GenomeFile.scala:
    239-249); a file it cannot parse falls back to the argument as a string."""
    names, lens = ["a", "b"], [1000, 500]
    f = tmp_path / "targets.txt"
    f.write_text("a:10-20,b\nb:5-6\n")
    assert parse_targets(str(f), names, lens) == [(0, 10, 20), (1, 1, 500), (1, 5, 6)]
    f.write_text("a:10-20\n\nb:5-6\n")  # a blank line fails the file; its name is no contig
    with pytest.raises(ValueError):
        parse_targets(str(f), names, lens)
    with pytest.raises(ValueError, match="within contig"):
        parse_targets("b:1-501", names, lens)
    assert contig_regions(1000, 300) == [(1, 250), (251, 500), (501, 750), (751, 1000)]


def test_unplaced_reads_at_the_end_are_left_out():
    """A coordinate-sorted BAM ends with its unplaced reads (reference -1, BAM
    position -1); no region query returns them, so the plan of a store with
    such a tail equals the plan without it, the last contig included.  A
    reference -1 read before placed reads is not coordinate order."""
    d = synth.generate(3, scale=0.005)
    lens = [c.size for c in d.contigs]
    rec = dict(pos=0, cigar=[], seq="ACGT" * 10, qual=[30] * 40, flag=4, mapq=0, ref_id=-1, mate_ref_id=-1)
    tail = build_store([rec] * 7)
    tail.aend = np.zeros(7, np.int32)
    plain = plan_regions(d.reads, lens, chunk_size=5000)
    assert plan_regions(concat_stores([d.reads, tail]), lens, chunk_size=5000) == plain
    last = [r for r in plain if r[0] == len(lens) - 1]
    assert last and all(b > a for (_, _, _, a, b) in last)
    with pytest.raises(ValueError, match="coordinate-sorted"):
        plan_regions(concat_stores([tail, d.reads]), lens, chunk_size=5000)


def test_merged_stores_give_the_same_pileups():
    """Two BAMs of one type merged into one coordinate-sorted store pile up as
    Pilon's sequential per-BAM processing does: the oracle over the merged store
    equals the oracle over the two stores one after the other (it scans a
    region's reads linearly, in any order)."""
    from oracle import oracle
    from pilon_gb300 import _abi
    from pilon_gb300.reads import merge_sorted
    d = synth.generate(1)
    r = d.reads
    a, b = r.subset(np.arange(0, r.n_reads, 2)), r.subset(np.arange(1, r.n_reads, 2))
    m = merge_sorted([a, b])
    seq = concat_stores([a, b])
    assert np.array_equal(m.pos, np.sort(r.pos, kind="stable")) and m.n_reads == r.n_reads
    L = d.contigs[0].size
    p = _abi.default_params()
    x = oracle.process_region(m, p, d.contigs[0], 0, 1, L)
    y = oracle.process_region(seq, p, d.contigs[0], 0, 1, L)
    for f in ("count", "qual_sum", "mq_sum", "q_sum", "phys_cov", "insert_size", "deletions", "insertions", "call",
              "score", "indel_len"):
        assert np.array_equal(getattr(x, f), getattr(y, f)), f
    assert x.stats.read_count == y.stats.read_count and x.stats.fr_sum == y.stats.fr_sum
