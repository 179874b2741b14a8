"""Local reassembly (fix types gaps and local) on the CPU: the host half of the
product path — BamFile.scan statistics and stray mates, GapFiller's read
recruitment (pilon_gb300/reassembly.py), the graph walk and GapFiller in C++
(pg_reassemble), and their fixes in the FASTA, changes and VCF
(pilon_gb300/polish.py) — against the oracle's restatement of
identifyAndFixIssues with gaps and local (S/GenomeRegion.scala:307-414,
S/GapFiller.scala:28-402, S/Assembler.scala:46-284).

The K-mer tally of each window is the device's job (pg_kmer_tally_reads,
compared in tests/test_gpu_reassembly.py); here the test-only stand-in engine
answers it from the oracle's tally of the same reads.
"""
import numpy as np
import pytest

from oracle import oracle
from pilon_gb300 import _abi, reassembly, synth
from pilon_gb300.engine import reassemble
from pilon_gb300.reads import build_store
from tests.test_polish_host import compare


@pytest.fixture(scope="module")
def cfg4_small():
    return synth.generate(4, 0.01)


def _big_fixes(changes):
    out = []
    for line in changes.decode().splitlines():
        was, patch = line.split()[2:4]
        was, patch = was.strip("."), patch.strip(".")
        if max(len(was), len(patch)) > 10:
            out.append(line)
    return out


@pytest.mark.parametrize("K", [31, 47])
def test_local_reassembly_matches_oracle(cfg4_small, K):
    """--fix all on 1.2 Mb with repeats and 10-200 bp planted indels: FASTA,
    changes and VCF byte-identical to the oracle, with local reassemblies."""
    n, out = compare(cfg4_small, vcf=True, fix_gaps=True, fix_local=True, K=K)
    big = _big_fixes(out["changes"])
    assert len(big) >= 10, big
    # the records of fixes only reassembly made (pileup indels keep their own records)
    assert out["vcf"].count(b"SVTYPE=INS") + out["vcf"].count(b"SVTYPE=DEL") >= 3


def test_variant_mode_opens_breaks(cfg4_small):
    """--variant adds the experimental "breaks" fix: a break that no join
    closes, away from a tandem repeat, is opened with each side's consensus and
    ten Ns (S/GapFiller.scala:76-99, S/Pilon.scala:232-236)."""
    n, out = compare(cfg4_small, vcf=True, fix_local=True, fix_breaks=True, K=31)
    assert any("N" in l.split()[3] for l in out["changes"].decode().splitlines())


def test_local_reassembly_without_strays(cfg4_small):
    compare(cfg4_small, vcf=True, fix_local=True, K=31, strays=False)


def test_jumps_recruit_bad_mates(cfg4_small):
    """A jumps BAM recruits the mates of its improper pairs' anchors
    (recruitBadMates, S/BamFile.scala:366-403) instead of the flank reads."""
    params = _abi.default_params(bam_type=_abi.PG_BAM_JUMPS)
    b = reassembly.BamState(cfg4_small.reads, params, 1)
    r = cfg4_small.reads
    lists = [b.recruit(0, s, s + 200) for s in range(20_000, 1_100_000, 50_000)]
    assert sum(x.size for x in lists) > 0
    for x in lists:
        assert np.all((r.flag[x] & 0x2) == 0)  # only improper pairs' ends
    compare(cfg4_small, params=params, vcf=True, fix_local=True, fix_gaps=True, K=31)


def test_reassemblies_restore_the_sample(cfg4_small):
    """Ground truth beside the oracle: the planted indels of 10 bp or more that
    local reassembly fixes leave the sample's own sequence in the polished
    FASTA around them.  Without --fix indels: a long indel that the pileup
    calls too would otherwise be inserted twice, at loci a few bases apart
    that fixFixList does not see as overlapping (S/GenomeRegion.scala:557-593),
    as in the reference."""
    d = cfg4_small
    n, out = compare(d, fix_local=True, fix_indels=False, K=31)
    fasta = b"".join(out["fasta"].split(b"\n")[1:])
    ref = bytes(d.contigs[0])
    fixed = restored = 0
    for line in _big_fixes(out["changes"]):
        loc = int(line.split()[0].split(":")[1].split("-")[0])
        near = [v for v in d.variants[0] if v[1] != "snp" and abs(v[0] - loc) < 300 and
                max(len(v[2]), len(v[3])) >= 10]
        if len(near) != 1:
            continue
        p, kind, was, alt = near[0]
        fixed += 1
        if kind == "ins":  # inserted after locus p
            sample = ref[p - 60:p] + alt.encode() + ref[p:p + 60]
        else:  # loci p .. p + len(was) - 1 deleted
            sample = ref[p - 61:p - 1] + ref[p - 1 + len(was):p - 1 + len(was) + 60]
        restored += sample in fasta
    assert fixed >= 10 and restored == fixed, (fixed, restored)


def test_gaps_closed_and_opened(cfg4_small):
    """GapFiller.fillGap on runs of N planted in the reference over sampled
    sequence: a 60 bp gap the reads span is closed with the sample's bases; a
    3 kb gap whose middle kilobase no read covers is filled from both sides
    with Ns between (S/GapFiller.scala:76-99)."""
    import copy
    d = copy.copy(cfg4_small)
    ref = d.contigs[0].copy()
    truth = bytes(ref[199_990:200_070])
    ref[200_000:200_060] = ord("N")
    ref[500_000:503_000] = ord("N")
    d.contigs = [ref]
    r = d.reads
    d.reads = r.subset(np.nonzero((r.aend < 501_000) | (r.pos > 502_000))[0])
    assert reassembly.gaps(ref, 1, ref.size) == [(200001, 200060), (500001, 503000)]
    for K in (31, 47):
        n, out = compare(d, vcf=True, fix_gaps=True, fix_local=True, K=K)
        lines = out["changes"].decode().splitlines()
        closed = [l for l in lines if l.startswith("chr1:200001-200060 ")]
        opened = [l for l in lines if l.split()[0].startswith("chr1:5000") and "N" in l.split()[3]]
        assert len(closed) == 1 and "N" not in closed[0].split()[3]
        assert len(opened) == 1 and len(opened[0].split()[3].strip("N")) > 0
        fasta = b"".join(out["fasta"].split(b"\n")[1:])
        assert truth in fasta


def test_gap_margin_and_min_gap(cfg4_small):
    """--gapmargin and --mingap (S/GapFiller.scala:69-73, 92): with a margin
    of -1 even the closed 60 bp gap (closed length 60, gap 60, difference 0)
    is refused and falls to the partial fill, and a minimum of 2,000 Ns
    widens the opened 3 kb gap's Ns to at least 2,000; both against the
    oracle with the same options."""
    import copy
    d = copy.copy(cfg4_small)
    ref = d.contigs[0].copy()
    ref[200_000:200_060] = ord("N")
    ref[500_000:503_000] = ord("N")
    d.contigs = [ref]
    r = d.reads
    d.reads = r.subset(np.nonzero((r.aend < 501_000) | (r.pos > 502_000))[0])

    def patches(out, first):
        return [l.split()[3] for l in out["changes"].decode().splitlines() if l.split()[0].startswith(first)]

    _, base = compare(d, fix_gaps=True, K=31)
    _, wide = compare(d, fix_gaps=True, K=31, min_gap=2000)
    _, tight = compare(d, fix_gaps=True, K=31, gap_margin=-1)
    assert patches(base, "chr1:200001-200060") and "N" not in patches(base, "chr1:200001-200060")[0]
    assert all("N" in p for p in patches(tight, "chr1:200001-200060"))
    opened_base = [p for p in patches(base, "chr1:5000") if "N" in p]
    opened_wide = [p for p in patches(wide, "chr1:5000") if "N" in p]
    assert len(opened_base) == 1 and len(opened_wide) == 1
    assert opened_base[0].count("N") < 2000 <= opened_wide[0].count("N")


def test_scan_statistics_and_strays(cfg4_small):
    """BamFile.scan over the store: the insert statistics and the stray-mate
    maps (one read per name and mate end) the recruitment looks mates up in."""
    d = cfg4_small
    P = _abi.default_params()
    b = reassembly.BamState(d.reads, P, 1)
    r = d.reads
    ok = reassembly.validate(r.flag, P) & ((r.flag & 0x4) == 0)
    proper = ok & ((r.flag & 0x3) == 0x3)
    t = r.tlen[proper].astype(np.int64)
    rc = (r.flag[proper] & 0x10) != 0
    keep = (t > 0) & (t < 2500)
    assert b.fr.count + b.rf.count == int(keep.sum())
    assert b.fr.sum == int(t[keep & ~rc].sum())
    assert 0 < b.max_insert_size() < 2500 and b.break_radius(47) >= 141
    strays = ok & ((r.flag & 0x3) == 0x1)
    n1, n2 = (b._stray[0][0].size, b._stray[1][0].size)
    assert n1 + n2 == int(strays.sum()) > 0
    # a window near a stray pair with one mate outside it recruits the other mate
    s_idx = np.nonzero(strays)[0]
    i = int(s_idx[len(s_idx) // 2])
    mate = int(s_idx[(r.name_id[s_idx] == r.name_id[i]) & (s_idx != i)][0])
    lo, hi = sorted((i, mate))
    flank = b.max_insert_size()
    win = b.recruit(0, int(r.pos[lo]) + flank, int(r.pos[lo]) + flank)  # overlaps read lo only
    assert lo in win.tolist() or hi in win.tolist()
    assert lo in win.tolist() and hi in win.tolist()


def _tile(seq, length=60, step=3, name0=0):
    """Forward reads tiling `seq` at `step`, quality 30, unpaired."""
    recs = []
    for k, p in enumerate(range(0, len(seq) - length + 1, step)):
        recs.append(dict(pos=p + 1, cigar=[(length, "M")], seq=seq[p:p + length], qual=[30] * length, flag=0,
                         mapq=60, name=name0 + k))
    return recs


def _graph(seq, K, **kw):
    reads = build_store(_tile(seq, **kw))
    e = oracle.kmer_tally_wide(reads, _abi.default_params(), [(0, reads.n_reads)], K)
    return e


def _job(region, bs, be, radius, gap=False):
    b = np.frombuffer(region.encode(), np.uint8).copy()
    return dict(window=0, is_gap=int(gap), region_start=1, region_stop=len(region), break_start=bs, break_stop=be,
                break_radius=radius, bases=b, orig=b)


def test_walk_closes_a_break_known_answer():
    """A region missing 25 bases that the reads hold: the walk from the left
    flank runs through the reads' sequence into the right flank, the joins give
    one solution, and trimPatch leaves the 25-base insertion
    (S/GapFiller.scala:49-262, S/Assembler.scala:183-284)."""
    rng = np.random.default_rng(7)
    sample = "".join("ACGT"[x] for x in rng.integers(0, 4, 1200))
    region = sample[:600] + sample[625:]
    edges = _graph(sample, 31)
    [(start, was, patch, status, loop)] = reassemble(edges, 31, [_job(region, 580, 620, 200)])
    assert status == 0 and loop == 0
    assert was == "" and patch == sample[600:625] and start == 601


def test_walk_stops_at_a_tandem_repeat_known_answer():
    """A break inside a tandem repeat longer than the reads: the walk meets a
    K-mer it has seen, notes the loop (its period) and, Pilon.trSafe being on,
    the break gets no solution (S/Assembler.scala:173-234, S/GapFiller.scala:67)."""
    rng = np.random.default_rng(11)
    flank = lambda n: "".join("ACGT"[x] for x in rng.integers(0, 4, n))
    unit = "ACCGTTAGC"
    sample = flank(500) + unit * 40 + flank(500)
    edges = _graph(sample, 31)
    [(start, was, patch, status, loop)] = reassemble(edges, 31, [_job(sample, 600, 700, 300)])
    assert status == 0 and start == 0 and loop == len(unit)


def test_walk_edge_of_region_raises_like_the_reference():
    """A break whose left flank would start before the region: subString's
    require fails in the reference (an exception ends the run); the job
    reports PG_ERR_INDEX."""
    rng = np.random.default_rng(3)
    sample = "".join("ACGT"[x] for x in rng.integers(0, 4, 400))
    edges = _graph(sample, 31)
    [(start, was, patch, status, loop)] = reassemble(edges, 31, [_job(sample, 1, 20, 50)])
    assert status == _abi.PG_ERR_INDEX


def test_bam_read_names_pair_mates(cfg4_small, tmp_path):
    """Read names survive a BAM round trip as ids (mates share one), so a store
    read from a BAM recruits the same stray mates as the simulator's store."""
    from pilon_gb300 import bam
    d = cfg4_small
    path = str(tmp_path / "reads.bam")
    bam.write_bam(path, d.names, [c.size for c in d.contigs], d.reads)
    _, _, st = bam.read_bam(path, names=True)
    a, b = d.reads.name_id, st.name_id
    # the same partition of reads into names
    assert np.unique(np.stack([a, b], 1), axis=0).shape[0] == np.unique(a).size == np.unique(b).size
    P = _abi.default_params()
    x, y = reassembly.BamState(d.reads, P, 1), reassembly.BamState(st, P, 1)
    for s in range(30_000, 1_100_000, 70_000):
        assert np.array_equal(x.recruit(0, s, s + 300), y.recruit(0, s, s + 300))
    _, _, plain = bam.read_bam(path)
    assert plain.name_id is None


def test_reassemble_arguments_and_empty_graphs():
    """pg_reassemble refuses bad jobs with PG_ERR_ARG, and a window without
    edges (no K-mer reached depth 5) gives no solution, like an Assembler
    whose graph is empty (S/Assembler.scala:183-190)."""
    import ctypes as C
    from pilon_gb300.engine import EngineError, lib
    rng = np.random.default_rng(5)
    region = "".join("ACGT"[x] for x in rng.integers(0, 4, 900))
    none = np.zeros(0, _abi.kmer_edge_wide_dtype())
    [(start, was, patch, status, loop)] = reassemble(none, 47, [_job(region, 400, 450, 150)])
    assert (start, status, loop) == (0, 0, 0)
    # a gap with an empty graph: both sides' consensus is its anchor, which matches the
    # region, so no partial fill either (partialMatchesReference)
    [(start, was, patch, status, loop)] = reassemble(none, 47, [_job(region, 400, 450, 150, gap=True)])
    assert (start, status) == (0, 0)
    with pytest.raises(EngineError):
        reassemble(none, 64, [_job(region, 400, 450, 150)])
    bad = _job(region, 400, 450, 150)
    bad["break_start"], bad["break_stop"] = 450, 400
    with pytest.raises(EngineError):
        reassemble(none, 47, [bad])
    with pytest.raises(ValueError):
        j = _job(region, 400, 450, 150)
        j["bases"] = j["bases"][:-1]
        reassemble(none, 47, [j])
    L = lib()
    n = C.c_int64()
    assert L.pg_reassemble(None, 0, 31, None, 0, 0, None, None, 0, C.byref(n)) == 0 and n.value == 0
    assert L.pg_reassemble(None, 0, 31, None, 1, 0, None, None, 0, C.byref(n)) == _abi.PG_ERR_ARG


@pytest.mark.parametrize("K", [31, 47, 63])
def test_walk_closes_a_break_for_each_K(K):
    """The known-answer insertion of test_walk_closes_a_break_known_answer at
    K = 31, 47 and 63 (the 4-bit keys span one to four words)."""
    rng = np.random.default_rng(7)
    sample = "".join("ACGT"[x] for x in rng.integers(0, 4, 1200))
    region = sample[:600] + sample[625:]
    edges = _graph(sample, K, length=100, step=2)
    [(start, was, patch, status, loop)] = reassemble(edges, K, [_job(region, 580, 620, 3 * K)])
    assert status == 0 and loop == 0
    assert was == "" and patch == sample[600:625] and start == 601


def test_gap_filled_with_the_reads_sequence_known_answer(tmp_path):
    """Worked by hand from S/GapFiller.scala:49-262: reads tiling a 2 kb sample
    aligned onto a reference that has its bases 900-959 replaced by N.  Pass 1
    skips the N positions; fillGap walks from the 93 bases before the gap
    (breakRadius = 3K for K = 31 without pairs) through the reads' K-mers, the
    join trims to the 60 bases under the Ns, and the gap closes with exactly
    the sample's bases: the polished FASTA is the sample, one changes line, and
    a reassembly VCF record of SVLEN 0 (written as INS)."""
    from types import SimpleNamespace
    from tests.test_oracle_kat import ref_from
    rng = np.random.default_rng(21)
    sample = "".join("ACGT"[x] for x in rng.integers(0, 4, 2000))
    ref = sample[:899] + "N" * 60 + sample[959:]
    recs = _tile(sample, length=100, step=5)
    ds = SimpleNamespace(names=["chr1"], contigs=[ref_from(ref)], reads=build_store(recs))
    n, out = compare(ds, vcf=True, fix_gaps=True, K=31)
    fasta = b"".join(out["fasta"].split(b"\n")[1:])
    assert fasta == sample.encode()
    assert out["changes"].decode() == f"chr1:900-959 chr1_pilon:900-959 {'N' * 60} {sample[899:959]}\n"
    fix = [l for l in out["vcf"].decode().splitlines() if "SVTYPE" in l and not l.startswith("#")]
    assert fix == [f"chr1\t899\t.\t{sample[898]}{'N' * 60}\t{sample[898:959]}\t.\tPASS\tSVTYPE=INS;SVLEN=0;"
                   f"END=959\tGT\t1/1"]


def test_break_reassembled_over_clipped_reads_known_answer():
    """A 30-base insertion that the aligner left as soft clips (reads are
    aligned up to the insertion and clipped after it, or clipped before it and
    aligned after): the clips mark a possible break (highClipping,
    S/GenomeRegion.scala:705-720), and fixBreak's walk through the reads'
    K-mers, clipped bases included, joins the flanks across it
    (S/GapFiller.scala:49-262): the polished sequence is the sample's."""
    from types import SimpleNamespace
    from tests.test_oracle_kat import ref_from
    rng = np.random.default_rng(33)
    ref = "".join("ACGT"[x] for x in rng.integers(0, 4, 3000))
    ins = "".join("ACGT"[x] for x in rng.integers(0, 4, 30))
    at = 1500  # the insertion follows reference base 1500 (1-based)
    sample = ref[:at] + ins + ref[at:]
    L, recs = 100, []
    for k, p in enumerate(range(0, len(sample) - L + 1, 3)):  # p: 0-based start in the sample
        seq = sample[p:p + L]
        if p + L <= at:  # left of the insertion
            cig, pos = [(L, "M")], p + 1
        elif p >= at + len(ins):  # right of it
            cig, pos = [(L, "M")], p - len(ins) + 1
        elif p < at:  # aligned up to the insertion, clipped after
            cig, pos = [(at - p, "M"), (L - (at - p), "S")], p + 1
        else:  # starts inside the insertion: clipped up to its end, aligned after
            c = at + len(ins) - p
            cig, pos = [(c, "S"), (L - c, "M")], at + 1
        recs.append(dict(pos=pos, cigar=cig, seq=seq, qual=[30] * L, flag=0, mapq=60, name=k))
    recs.sort(key=lambda r: r["pos"])
    ds = SimpleNamespace(names=["chr1"], contigs=[ref_from(ref)], reads=build_store(recs))
    n, out = compare(ds, vcf=True, fix_local=True, fix_indels=False, K=31)
    fasta = b"".join(out["fasta"].split(b"\n")[1:])
    assert fasta == sample.encode()
    lines = out["changes"].decode().splitlines()
    assert len(lines) == 1 and lines[0].split()[2] == "." and len(lines[0].split()[3]) == len(ins)


def test_local_reassembly_many_contigs():
    """--fix all over 15 uneven contigs of the draft workload (1% of bases
    carry SNPs and indels): every contig's regions see the insert statistics
    of the scan and of the regions before them (H7)."""
    ds = synth.generate(3, scale=0.005)
    n, out = compare(ds, vcf=True, fix_gaps=True, fix_local=True, K=31)
    assert n > 100


def test_scan_reads_matches_numpy_restatement():
    """pg_scan_reads against BamFile.scan restated in numpy on a store of
    random flags, insert sizes, lengths and references: the nine insert
    statistics (sumSq wrapping as a Scala Int) and the stray-mate indices, for
    each BAM type's size cut and with --nonpf / --duplicates."""
    from pilon_gb300.engine import scan_reads
    rng = np.random.default_rng(21)
    n = 200_000
    recs = dict(flag=rng.integers(0, 1 << 12, n).astype(np.uint16),
                tlen=rng.integers(-60_000, 60_000, n).astype(np.int32),
                l_seq=rng.integers(0, 60_000, n).astype(np.int32),
                ref_id=rng.integers(-1, 4, n).astype(np.int32), mate_ref_id=rng.integers(-1, 4, n).astype(np.int32))

    class Store:  # the fields pg_scan_reads reads; the others empty
        n_reads = n

        def to_abi(self):
            r = _abi.pg_reads()
            r.n_reads = n
            self._keep = recs
            for k, v in recs.items():
                setattr(r, k, v.ctypes.data)
            return r

    for nonpf, dups, bam_type in ((0, 0, _abi.PG_BAM_FRAGS), (1, 0, _abi.PG_BAM_JUMPS), (0, 1, _abi.PG_BAM_UNPAIRED)):
        P = _abi.default_params(nonpf=nonpf, duplicates=dups, bam_type=bam_type)
        huge = 5 * reassembly.MAX_INSERT_DEFAULT[bam_type]
        stats, first, second = scan_reads(Store(), P, 3, huge, strays=True, threads=3)
        f = recs["flag"]
        ok = reassembly.validate(f, P) & ((f & 0x4) == 0)
        paired, proper, rc = (f & 1) != 0, (f & 2) != 0, (f & 0x10) != 0
        want = []
        for sizes, sel in ((recs["tlen"], ok & paired & proper & ~rc), (recs["tlen"], ok & paired & proper & rc),
                           (recs["l_seq"], ok & ~paired)):
            s = sizes[sel].astype(np.int64)
            s = s[(s > 0) & (s < huge)]
            want += [s.size, int(s.sum()), int((s * s).astype(np.int32).sum(dtype=np.int64))]
        assert stats.tolist() == want
        rid, mrid = recs["ref_id"], recs["mate_ref_id"]
        soi = ((rid >= 0) & (rid < 3)) | ((mrid >= 0) & (mrid < 3))
        st = ok & paired & ~proper & ((f & 0x8) == 0) & soi
        idx = np.nonzero(st)[0]
        assert first.tolist() == idx[(f[idx] & 0x40) != 0].tolist()
        assert second.tolist() == idx[(f[idx] & 0x40) == 0].tolist()
        stats2, f2, s2 = scan_reads(Store(), P, 3, huge, strays=False)
        assert stats2.tolist() == want and f2.size == s2.size == 0
