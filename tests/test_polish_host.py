"""The host side of pilon_gb300.polish on the CPU: fix lists, the AMB options,
fixFixList, fixIssues, the changes offsets across region chunks and the FASTA
(S/GenomeRegion.scala:307-414, 557-657, S/GenomeFile.scala:135-161).

A test-only stand-in answers the engine calls polish() makes (set_reference,
set_reads, pileup_regions, stats and the pg_fetch_region ctypes call) from the
oracle's per-region results; the FASTA and changes files polish() writes must
then equal the oracle's own restatement of GenomeFile.processRegions byte for
byte.  The per-position VCF records are the engine's device formatter's (compared
in the GPU tests); here the stand-in cuts them from the oracle's VCF, so a VCF
comparison checks what polish() adds: the header, copy number and <DUP> records.
"""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

from oracle import oracle
from pilon_gb300 import _abi, synth
from pilon_gb300.polish import Options, polish

FIELDS = ["count", "qual_sum", "mq_sum", "q_sum", "phys_cov", "insert_size", "bad_pair", "deletions", "del_qual",
          "insertions", "ins_qual", "clips", "call", "score", "indel_len", "ins_str"]


class _OracleFetch:
    """pg_fetch_region's contract (include/pilon_gb300.h) over an oracle result:
    fills every non-NULL field; with ins_chars NULL it only reports the pool's
    size in ins_chars_cap, else it copies the pool when it fits."""

    def __init__(self, owner):
        self.owner = owner

    def pg_fetch_region(self, h, r, oref):
        o = oref._obj
        res = self.owner.results[r]
        for f in FIELDS:
            dst = getattr(o, f)
            if dst:
                a = np.ascontiguousarray(getattr(res, f))
                C.memmove(dst, a.ctypes.data, a.nbytes)
        ins = np.nonzero(res.ins_str >= 0)[0]
        used = int((res.ins_str[ins].astype(np.int64) + res.indel_len[ins]).max()) if ins.size else 0
        if o.ins_chars:
            if used > o.ins_chars_cap:
                return _abi.PG_ERR_LIMIT
            C.memmove(o.ins_chars, res.ins_chars.ctypes.data, used)
        o.ins_chars_cap = used
        return _abi.PG_OK


class OracleEngine:
    """Test-only stand-in for pilon_gb300.engine.Engine, backed by the oracle.
    format_vcf returns a region's records cut from the oracle's own VCF of the
    same store (a region's records all have POS inside it), without the <DUP>
    records, which polish() splices in itself."""
    h = None

    def __init__(self, names=None, chunk=10_000_000, **fix):
        self.L = _OracleFetch(self)
        self.names, self.chunk, self._vcf = names, chunk, {}
        self.fix = fix  # fix_gaps / fix_local / K / strays of the oracle run the VCF records come from

    def set_reference(self, contigs):
        self.contigs = contigs

    def set_reads(self, reads):
        self.reads = reads

    def pileup_regions(self, regions, params, batched=True):
        self.regions, self.params = regions, params
        self.results = [oracle.process_region(self.reads, params, self.contigs[c], c, s, e, rb, re)
                        for (c, s, e, rb, re) in regions]
        assert all(r.status == 0 for r in self.results)

    def stats(self, r):
        return self.results[r].stats

    def fetch_changes(self):
        """pg_fetch_changes' contract over the oracle's per-region arrays: the
        changed positions of every region in locus order, with insertion offsets
        into one pool of all regions' insertion characters."""
        rows, pool = [], b""
        for r, (c, s, e, rb, re) in enumerate(self.regions):
            res = self.results[r]
            for i in np.nonzero((res.call >> 9) & 7)[0].tolist():
                off = -1
                if int(res.ins_str[i]) >= 0:
                    off = len(pool)
                    pool += res.insertion(i).encode()
                rows.append((r, s + i, int(res.call[i]), int(res.indel_len[i]), off, 0))
        return np.array(rows, dtype=_abi.change_dtype()), pool

    def find_duplications(self):
        """duplicationEvents restated on the host from the oracle's arrays: pass 2
        of postProcess (smooth, copyNumber) and summaryRegions, as the device's
        pg_find_duplications computes them."""
        from tests.breaks_host import java_round, smooth, summary_regions
        out = {}
        for r, (c, s, e, rb, re) in enumerate(self.regions):
            res = self.results[r]
            if res.stats.read_count <= 0:
                continue
            size = e - s + 1
            # fragCoverage = depth after the BAM, before pass 1 added deletion counts
            frag = res.count.reshape(-1, 4).astype(np.int64).sum(1) + res.deletions
            for i in np.nonzero(((res.call >> 9) & 7) == _abi.PG_CHANGE_DEL)[0].tolist():
                frag[i + 1:i + int(res.indel_len[i])] -= int(res.deletions[i])
            mean = float(frag.sum()) / size
            sm = smooth(frag, 200)
            cn = java_round(sm / mean) if mean > 0 else np.zeros(size, np.int64)
            d = [x for x in summary_regions(cn > 1, s, e, 2000) if x[1] + 1 - x[0] > 10000]
            if d:
                out[r] = d
        return out

    def find_breaks(self, min_min_depth=5):
        """possibleBreaks of every region, from the oracle (pg_find_breaks)."""
        out = {}
        for r, (c, s, e, rb, re) in enumerate(self.regions):
            b = oracle.region_breaks(self.reads, self.params, self.contigs[c], c, s, e, rb, re)
            if b:
                out[r] = b
        return out

    def kmer_tally_reads(self, read_lists, K, params, min_depth=5):
        """pg_kmer_tally_reads' edges from the oracle's tally of each list."""
        parts = []
        for w, lst in enumerate(read_lists):
            sub = self.reads.subset(np.asarray(lst, np.int64))
            e = oracle.kmer_tally_wide(sub, params, [(0, sub.n_reads)], K, min_depth)
            e["window"] = w
            parts.append(e)
        return np.concatenate(parts) if parts else np.zeros(0, _abi.kmer_edge_wide_dtype())

    def mark_deleted(self, r, first_locus, count):
        s = self.regions[r][1]
        self.results[r].call[first_locus - s:first_locus - s + count] |= _abi.PG_CALL_DELETED

    def _check(self, st):
        assert st == _abi.PG_OK, st

    def format_vcf(self, r, name, diploid, vcf_qe, variants_only=False):
        assert not variants_only
        key = (bool(diploid), bool(vcf_qe))
        if key not in self._vcf:
            with tempfile.TemporaryDirectory() as d:
                pre = os.path.join(d, "v")
                assert oracle.polish(self.reads, self.params, self.names, self.contigs, pre, chunk_size=self.chunk,
                                     diploid=diploid, vcf_qe=vcf_qe, **self.fix) == 0
                body = [l for l in open(pre + ".vcf", "rb").read().split(b"\n") if l and not l.startswith(b"#")]
            by_contig = {}
            for l in body:
                f = l.split(b"\t", 8)
                if f[4] != b"<DUP>" and not f[7].startswith(b"SVTYPE="):  # not a <DUP> or reassembly record
                    lines, locs = by_contig.setdefault(f[0], ([], []))
                    lines.append(l)
                    locs.append(int(f[1]))
            self._vcf[key] = by_contig
        import bisect
        s, e = self.regions[r][1:3]
        lines, locs = self._vcf[key].get(name.encode(), ([], []))
        out = lines[bisect.bisect_left(locs, s):bisect.bisect_right(locs, e)]
        return b"".join(l + b"\n" for l in out)


def compare(ds, params=None, chunk=10_000_000, no_frags=False, vcf=False, **kw):
    params = params or _abi.default_params()
    opts = Options(chunk_size=chunk, vcf=vcf, **kw)
    opts.no_frags = no_frags  # long reads only: excludeMotifs applies
    fix = dict(fix_gaps=opts.fix_gaps, fix_local=opts.fix_local, K=opts.K, strays=opts.strays,
               fix_breaks=opts.fix_breaks, gap_margin=opts.gap_margin, min_gap=opts.min_gap)
    with tempfile.TemporaryDirectory() as d:
        h, o = os.path.join(d, "host"), os.path.join(d, "ora")
        polish(OracleEngine(ds.names, chunk, **fix), ds.names, ds.contigs, ds.reads, params, h, opts)
        assert oracle.polish(ds.reads, params, ds.names, ds.contigs, o, chunk_size=chunk, fix_snps=opts.fix_snps,
                             fix_indels=opts.fix_indels, iupac=opts.iupac, diploid=opts.diploid,
                             vcf_qe=opts.vcf_qe, vcf_date=opts.vcf_date, vcf_source=opts.vcf_source,
                             vcf_args=opts.vcf_args, vcf_ref=opts.vcf_ref, **fix) == 0
        out = {}
        for ext in ("fasta", "changes") + (("vcf",) if vcf else ()):
            a, b = open(f"{h}.{ext}", "rb").read(), open(f"{o}.{ext}", "rb").read()
            assert a == b, ext
            out[ext] = a
        return out["changes"].count(b"\n"), out


def test_defaults(cfg1):
    assert compare(cfg1)[0] >= 20


@pytest.mark.parametrize("kw,pk", [(dict(chunk=9000, iupac=True), dict(fix_amb=1)),
                                   (dict(chunk=20000), dict(fix_amb=1)),
                                   (dict(fix_indels=False), {}),
                                   (dict(fix_snps=False), {})])
def test_options_and_chunks(cfg1, kw, pk):
    compare(cfg1, params=_abi.default_params(**pk), **kw)


def test_many_contigs():
    compare(synth.generate(3, scale=0.01))


@pytest.mark.parametrize("ref_base,kw,pk", [("G", {}, {}), ("G", dict(iupac=True), {}), ("C", {}, {}),
                                            ("C", dict(iupac=True), dict(fix_amb=1))])
def test_ambiguous_fixes(ref_base, kw, pk):
    """The AMB branches (base or IUPAC code, --fix amb) on the hand-worked
    6A/4C position, which the synthetic workloads do not produce."""
    from types import SimpleNamespace
    from pilon_gb300.reads import build_store
    from tests.test_oracle_kat import _het_reads, rand_ref, ref_from
    ref = list(rand_ref(100, seed=5))
    ref[49] = ref_base
    ref = "".join(ref)
    ds = SimpleNamespace(names=["chr1"], contigs=[ref_from(ref)], reads=build_store(_het_reads(ref)))
    n, _ = compare(ds, params=_abi.default_params(**pk), **kw)
    assert n == (1 if ref_base == "G" or pk else 0)


@pytest.mark.parametrize("snp_locus", [61, 62, 40])
def test_long_read_only_motif_exclusion(snp_locus):
    """excludeMotifs with long reads only (run starts of 4+ bases are not fixed),
    on the hand-worked A run at loci 60-64."""
    from types import SimpleNamespace
    from pilon_gb300.reads import build_store
    from tests.test_oracle_kat import _tile_reads, rand_ref, ref_from
    ref = list(rand_ref(120, seed=43))
    ref[58], ref[59:64], ref[64] = "C", "AAAAA", "G"
    ref = "".join(ref)
    snp = "T" if ref[snp_locus - 1] != "T" else "G"
    recs, _ = _tile_reads(ref, snps={snp_locus: snp}, length=40, step=1)
    ds = SimpleNamespace(names=["chr1"], contigs=[ref_from(ref)], reads=build_store(recs))
    params = _abi.default_params(long_read=_abi.PG_PACBIO, long_read_only=1)
    n, _ = compare(ds, params=params, longread=True, no_frags=True)
    assert n == (0 if snp_locus == 61 else 1)


def test_vcf_header_and_duplication_record():
    """The VCF header and the <DUP> record of copy number 2 over a 14 kb stretch
    read twice (GenomeRegion copy number and writeDup, S/GenomeRegion.scala:
    272-283, 623-631, S/Vcf.scala:28-68, 194-202), with the per-position records
    taken from the oracle."""
    w = synth.workload(1, scale=1.2)
    ds = synth.generate(w)
    r = ds.reads
    sel = np.nonzero((r.pos > 20_000) & (r.aend < 34_000))[0]
    ds.reads = r.subset(np.sort(np.concatenate([np.arange(r.n_reads), sel]), kind="stable"))
    _, out = compare(ds, vcf=True)
    dup = [l for l in out["vcf"].split(b"\n") if b"<DUP>" in l]
    assert len(dup) == 1 and b"SVTYPE=DUP" in dup[0]
    compare(ds, vcf=True, chunk=25_000, vcf_qe=True, diploid=True)


def test_targets_are_separate_outputs():
    """--targets makes every target its own entry of GenomeFile.regions
    (S/GenomeFile.scala:49-54, 215-236), and the writers loop over those entries
    (S/GenomeFile.scala:135-161): two targets on one contig give two FASTA
    records of their fixed bases, and the second target's changes are not
    shifted by the first one's insertion (the offset restarts per entry)."""
    from types import SimpleNamespace
    from pilon_gb300.reads import build_store
    from tests.test_oracle_kat import _tile_reads, rand_ref, ref_from
    ref = list(rand_ref(2000, seed=51))
    if ref[308] == "A":  # locus 309 is not 'A': the insertion before 310 does not shift
        ref[308] = "G" if ref[307] != "G" and ref[309] != "G" else "T"
    ref = "".join(ref)
    s1 = "ACGT"[("ACGT".index(ref[299]) + 1) % 4]
    s2 = "ACGT"[("ACGT".index(ref[1499]) + 1) % 4]
    recs, _ = _tile_reads(ref, snps={300: s1, 1500: s2}, ins={310: "CA"})
    ds = SimpleNamespace(names=["chr1"], contigs=[ref_from(ref)], reads=build_store(recs))
    opts = Options(vcf=False, targets=[(0, 200, 800), (0, 1000, 1800)])
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "t")
        polish(OracleEngine(ds.names), ds.names, ds.contigs, ds.reads, _abi.default_params(), pre, opts)
        fa = open(pre + ".fasta").read()
        ch = open(pre + ".changes").read().splitlines()
    t1 = ref[199:299] + s1 + ref[300:309] + "CA" + ref[309:800]
    t2 = ref[999:1499] + s2 + ref[1500:1800]
    wrap = lambda s: "".join(s[k:k + 80] + "\n" for k in range(0, len(s), 80))
    assert fa == ">chr1_pilon\n" + wrap(t1) + ">chr1_pilon\n" + wrap(t2)
    assert ch == [f"chr1:300 chr1_pilon:300 {ref[299]} {s1}", "chr1:310 chr1_pilon:310-311 . CA",
                  f"chr1:1500 chr1_pilon:1500 {ref[1499]} {s2}"]


def test_contig_order_is_the_output_order():
    """Options.contig_order (the FASTA's order, pilon_gb300.fasta.reference_for_bam)
    sets the order contigs are processed and written in, as GenomeFile.regions
    follows the FASTA (S/GenomeFile.scala:49-54): reversing it reverses the FASTA
    records and the contigs' blocks of changes lines."""
    ds = synth.generate(3, scale=0.01)
    n = len(ds.contigs)
    outs = []
    for order in (None, list(range(n))[::-1]):
        with tempfile.TemporaryDirectory() as d:
            pre = os.path.join(d, "o")
            polish(OracleEngine(ds.names), ds.names, ds.contigs, ds.reads, _abi.default_params(), pre,
                   Options(vcf=False, contig_order=order))
            fa = open(pre + ".fasta").read().split(">")[1:]
            ch = open(pre + ".changes").read().splitlines()
        outs.append((fa, ch))
    (fa0, ch0), (fa1, ch1) = outs
    assert len(fa0) == n and fa1 == fa0[::-1]
    by_contig = lambda lines: [[l for l in lines if l.split(":")[0] == nm] for nm in ds.names]
    assert by_contig(ch1) == by_contig(ch0)
    assert [l.split(":")[0] for l in ch1] == sorted((l.split(":")[0] for l in ch0),
                                                    key=lambda nm: -ds.names.index(nm))


def test_soft_masked_reference():
    """A reference with a lowercase (soft-masked) stretch holding a SNP, an
    insertion and a deletion: the host driver's fixes and FASTA equal the
    oracle's, which keeps the file's case wherever nothing is fixed."""
    from types import SimpleNamespace
    from pilon_gb300.reads import build_store
    from tests.test_oracle_kat import _tile_reads, rand_ref, ref_from
    up = rand_ref(900, seed=61)
    snp = "ACGT"[("ACGT".index(up[299]) + 1) % 4]
    recs, _ = _tile_reads(up, snps={300: snp}, ins={501: "GT"}, dels={601: 602})
    ref = up[:200] + up[200:700].lower() + up[700:]
    ds = SimpleNamespace(names=["chr1"], contigs=[ref_from(ref)], reads=build_store(recs))
    n, out = compare(ds)
    assert n >= 2 and any(c.islower() for c in out["fasta"].decode())


@pytest.mark.parametrize("wl,kw,pk", [
    (2, dict(chunk=20000, iupac=True, vcf=True), dict(fix_amb=1, min_qual=20)),
    (2, dict(chunk=33333, fix_indels=False, diploid=True, vcf=True), dict(flank=25)),
    (2, dict(fix_snps=False), dict(min_mq=10, flank=0)),
    (3, dict(chunk=20000, vcf=True, vcf_qe=True), dict(fix_amb=1)),
    (3, dict(longread=True, nanopore=True), dict(long_read=_abi.PG_NANOPORE, bam_type=_abi.PG_BAM_UNPAIRED)),
    (3, dict(chunk=33333, longread=True, nanopore=False, vcf=True),
     dict(long_read=_abi.PG_PACBIO, bam_type=_abi.PG_BAM_UNPAIRED, min_qual=20)),
])
def test_option_combinations_on_other_workloads(wl, kw, pk):
    """The host driver against the oracle on the 100x workload with mapq-0
    reads and indel errors and on the many-contig workload (both scaled), over
    combinations of chunking, fix types, AMB options, read filters, flank,
    long-read modes and VCF flavours."""
    ds = synth.generate(wl, scale=0.01)
    compare(ds, params=_abi.default_params(**pk), **kw)


def request_result(engine, r, req, names, contigs, params, opts):
    """One served answer restated on the host from region r of the last engine
    call: the fixed bases, the changes lines of the target as its own output
    entry (offset 0) and the variant records, as the native server builds them
    (pilon_gb300/csrc/pg_serve.cu)."""
    from pilon_gb300.polish import _region_outputs, new_name, region_string
    from pilon_gb300.serve import Result
    region = (req.contig, req.start, req.stop, 0, 0)
    changes, chars = engine.fetch_changes()
    res = _region_outputs(engine, r, region, contigs[req.contig], opts, params, changes[changes["region"] == r],
                          chars)
    nn = new_name(names[req.contig])
    lines = []
    delta = 0
    for f in res.all_fixes():
        nl = f.locus + delta
        lines.append(region_string(names[req.contig], f.locus, f.locus + len(f.was) - 1) + " " +
                     region_string(nn, nl, nl + len(f.patch) - 1) + " " + (f.was or ".") + " " + (f.patch or "."))
        delta += len(f.patch) - len(f.was)
    vcf = engine.format_vcf(r, names[req.contig], opts.diploid, opts.vcf_qe, variants_only=True)
    return Result(req.rid, bytes(res.bases), "".join(l + "\n" for l in lines), vcf)


def test_served_requests_equal_target_outputs():
    """A served answer, restated on the host (request_result), equals what
    --targets writes for that target: its fixed bases and its changes lines
    (each target its own entry, the offset restarting)."""
    from types import SimpleNamespace
    from pilon_gb300.reads import build_store
    from pilon_gb300.regions import plan_regions
    from pilon_gb300.serve import Request
    from tests.test_oracle_kat import _tile_reads, rand_ref, ref_from
    ref = list(rand_ref(2000, seed=51))
    if ref[308] == "A":
        ref[308] = "G" if ref[307] != "G" and ref[309] != "G" else "T"
    ref = "".join(ref)
    s1 = "ACGT"[("ACGT".index(ref[299]) + 1) % 4]
    s2 = "ACGT"[("ACGT".index(ref[1499]) + 1) % 4]
    recs, _ = _tile_reads(ref, snps={300: s1, 1500: s2}, ins={310: "CA"}, dels={1601: 1602})
    ds = SimpleNamespace(names=["chr1"], contigs=[ref_from(ref)], reads=build_store(recs))
    targets = [(0, 200, 800), (0, 1000, 1800)]
    opts = Options(vcf=False, targets=targets)
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "t")
        polish(OracleEngine(ds.names), ds.names, ds.contigs, ds.reads, _abi.default_params(), pre, opts)
        fasta = open(pre + ".fasta").read().split(">chr1_pilon\n")[1:]
        changes = open(pre + ".changes").read()
    eng = OracleEngine(ds.names)
    eng.set_reference(ds.contigs)
    eng.set_reads(ds.reads)
    eng.pileup_regions(plan_regions(ds.reads, [len(ref)], targets=targets), _abi.default_params())
    eng.format_vcf = lambda *a, **k: b""
    got_fa, got_ch = [], ""
    for r, (c, s, e) in enumerate(targets):
        res = request_result(eng, r, Request(contig=c, start=s, stop=e), ds.names, ds.contigs,
                             _abi.default_params(), Options(vcf=False))
        got_fa.append(res.fasta.decode() if isinstance(res.fasta, bytes) else res.fasta)
        got_ch += res.changes
    assert [f.replace("\n", "") for f in fasta] == got_fa
    assert got_ch == changes and changes.count("\n") == 4


def test_fix_issues_joined_matches_fixes_applied_in_turn():
    """fix_issues joins the unchanged stretches and the patches once; on random
    fix lists (SNPs, insertions, deletions, replacements, overlaps, several at
    one locus) the result is the one of applying the fixes one by one from the
    last locus, as GenomeRegion.fixIssues does (S/GenomeRegion.scala:595-621)."""
    from pilon_gb300.polish import Fix, _fix_issues_in_turn, fix_fix_list, fix_issues
    rng = np.random.default_rng(7)
    for trial in range(400):
        n = int(rng.integers(1, 60))
        start = int(rng.integers(1, 1000))
        bases = bytes(rng.choice(list(b"ACGT"), n).astype(np.uint8))
        fixes = []
        for _ in range(int(rng.integers(0, 8))):
            locus = start + int(rng.integers(0, n))
            kind = int(rng.integers(0, 4))
            wl = {0: 1, 1: 0, 2: int(rng.integers(1, 5)), 3: int(rng.integers(1, 4))}[kind]
            pl = {0: 1, 1: int(rng.integers(1, 5)), 2: 0, 3: int(rng.integers(1, 6))}[kind]
            was = bases[locus - start:locus - start + wl].decode()
            patch = "".join(rng.choice(list("ACGTN"), pl))
            fixes.append(Fix(locus, was, patch))
        want = _fix_issues_in_turn(bases, start, fix_fix_list(fixes))
        assert fix_issues(bases, start, fixes) == want, (trial, fixes)
        assert fix_issues(np.frombuffer(bases, np.uint8), start, fixes) == want
    # a fix before the region's start goes the step-by-step way
    fixes = [Fix(8, "", "GG"), Fix(12, "A", "T")]
    assert fix_issues(b"CCAAC", 10, fixes) == _fix_issues_in_turn(b"CCAAC", 10, fix_fix_list(fixes))


def test_fasta_lines_wraps_at_80():
    from pilon_gb300.polish import fasta_lines
    for n in (0, 1, 79, 80, 81, 159, 160, 161, 1000):
        seq = bytes(np.arange(n, dtype=np.uint8) % 26 + 65)
        want = b"".join(seq[k:k + 80] + b"\n" for k in range(0, n, 80))
        assert fasta_lines(seq) == want, n


def _exclude_motifs_by_locus(orig, nano):
    """excludeMotifs as the reference states it, locus by locus: homoRun walks
    right from each locus to the region's stop (S/GenomeRegion.scala:416-439)."""
    b = bytes(orig).upper()
    n = len(b)
    ex = []
    for i in range(n):
        run = 1
        while i + run < n and b[i + run] == b[i]:
            run += 1
        cc_gg = 2 <= i < n - 2 and b[i - 2:i] == b"CC" and b[i + 1:i + 3] == b"GG"
        ex.append(run >= 4 or (nano and cc_gg))
    return np.array(ex, bool)


def test_exclude_motifs_matches_homorun_by_locus():
    from pilon_gb300.polish import _exclude_motifs
    rng = np.random.default_rng(11)
    for n in (0, 1, 3, 4, 5, 6, 9, 40, 300):
        for _ in range(20):
            seq = bytes(rng.choice(list(b"CCGGAT"), n).astype(np.uint8)).lower() if rng.random() < 0.3 else \
                bytes(rng.choice(list(b"CCGGAT"), n).astype(np.uint8))
            for nano in (False, True):
                got = _exclude_motifs(seq, 1, n, nano)
                assert np.array_equal(got, _exclude_motifs_by_locus(seq, nano)), (seq, nano)
