"""Whole-genome polishing on the GB300 engine: the loop of
GenomeFile.processRegions (S/GenomeFile.scala:84-176) for the fix types
snps / indels (and amb / iupac) and gaps / local, writing Pilon's three
outputs.

  pileup, BaseCall, pass 1      engine (pg_pileup_regions), batched over all regions
  fix lists, fixIssues          host, over the sparse change list (S/GenomeRegion.scala:307-414, 557-621)
  gaps / local reassembly       reassembly.py: recruitment on the host, the K-mer tally of every
                                window on the device (pg_kmer_tally_reads), the graph walk and
                                GapFiller on host threads (pg_reassemble)
  VCF records                   engine (pg_format_vcf); header, <DUP> and reassembly records here
  changes, FASTA                host (S/GenomeRegion.scala:645-657, S/GenomeFile.scala:79-82, 135-161)
"""
import ctypes as C
import operator
from dataclasses import dataclass

import numpy as np

from . import _abi
from .engine import changes_lines, region_fixes
from .regions import plan_regions
from . import reassembly


@dataclass
class Options:
    """The command-line switches of Pilon that this path honours (S/Pilon.scala:28-73)."""
    fix_snps: bool = True
    fix_indels: bool = True
    fix_gaps: bool = False          # "gaps": GapFiller.fillGap over runs of N
    fix_local: bool = False         # "local": GapFiller.fixBreak over possibleBreaks
    fix_breaks: bool = False        # experimental "breaks" (--variant): unjoined breaks are opened
    K: int = 47                     # --K, Assembler.K
    strays: bool = True             # --nostrays clears it
    gap_margin: int = 100000        # --gapmargin: a closed gap may differ from the gap's length by this much
    min_gap: int = 10               # --mingap: the Ns a partial gap fill leaves at least
    iupac: bool = False
    diploid: bool = False
    vcf: bool = True
    vcf_qe: bool = False
    changes: bool = True
    longread: bool = False
    nanopore: bool = False
    chunk_size: int = 10_000_000
    targets: list = None            # [(contig, start, stop)] or None
    contig_order: list = None       # contig indices to process and write, in order (FASTA order); None = all
    vcf_date: str = "20260101"
    vcf_source: str = "Pilon version [COMMIT] [DATE]"
    vcf_args: str = ""
    vcf_ref: str = "file:/genome.fasta"


@dataclass
class Fix:
    locus: int
    was: str
    patch: str


def _locus(f):
    return f.locus


def fix_fix_list(fixes):
    """GenomeRegion.fixFixList (S/GenomeRegion.scala:557-593): stable sort by
    locus, then of two overlapping fixes keep the one with more bases.  After
    the sort a fix overlaps the next one when the next starts at or before
    its last replaced locus; a list without such a pair comes back as sorted."""
    fx = sorted(fixes, key=_locus)
    if len(fx) > 1:
        loci = [f.locus for f in fx]
        last = [f.locus + (len(f.was) - 1 if f.was else 0) for f in fx]
        if not any(map(operator.le, loci[1:], last[:-1])):
            return fx
    out = []
    k = 0
    while k < len(fx):
        if k + 1 < len(fx):
            f1, f2 = fx[k], fx[k + 1]
            e1 = f1.locus + max(len(f1.was) - 1, 0)
            e2 = f2.locus + max(len(f2.was) - 1, 0)
            if f2.locus <= e1 and e2 >= f1.locus:
                if len(f1.was) + len(f1.patch) >= len(f2.was) + len(f2.patch):
                    fx[k + 1] = f1
                k += 1
            else:
                out.append(f1)
                k += 1
        else:
            out.append(fx[k])
            k += 1
    return out


def fix_issues(bases, start, fixes):
    """GenomeRegion.fixIssues (S/GenomeRegion.scala:595-621) on a bytearray.

    Pilon applies the fixes from the last locus to the first, each on the
    original coordinates.  fixFixList leaves fixes whose replaced ranges follow
    one another, so that is the original bases between the ranges and each
    patch in order, joined once (linear in the region, where splicing each
    indel into the whole region is quadratic).  A fix that starts before the
    end of the one before it (only a locus before the region's start can) is
    applied the step-by-step way, as Pilon does."""
    fx = fix_fix_list(fixes)
    src = bytes(bases)
    parts, at = [], 0
    for f in fx:
        s = f.locus - start
        if s < at:
            return _fix_issues_in_turn(src, start, fx)
        parts.append(src[at:s])
        parts.append(f.patch.encode())
        at = s + len(f.was)
    parts.append(src[at:])
    return bytearray(b"".join(parts))


def _fix_issues_in_turn(bases, start, fx):
    """fixIssues step by step: the fixes of fx from the last to the first."""
    nb = bytearray(bases)
    for f in reversed(fx):
        s = f.locus - start
        if len(f.was) == len(f.patch):
            nb[s:s + len(f.patch)] = f.patch.encode()
        else:
            nb = nb[:s] + f.patch.encode() + nb[s + len(f.was):]
    return nb


def fasta_lines(seq, width=80):
    """A FASTA record's sequence lines (FastaWriter's 80 bases per line, the
    last line shorter), as one buffer with a newline after each line."""
    a = np.frombuffer(seq, np.uint8)
    n = a.size
    full = n // width
    out = np.empty(n + (n + width - 1) // width, np.uint8)
    body = out[:full * (width + 1)].reshape(full, width + 1)
    body[:, :width] = a[:full * width].reshape(full, width)
    body[:, width] = 10
    if n > full * width:
        out[full * (width + 1):-1] = a[full * width:]
        out[-1] = 10
    return out.tobytes()


def region_string(name, s, e):  # Region.regionString (S/Region.scala:45)
    return f"{name}:{s}" + ("" if e + 1 - s < 2 else f"-{e}")


class RegionResult:
    """One region's outputs: the fix lists of GenomeRegion (snpFixList and
    smallFixList from pass 1, bigFixList from local reassembly), its bases
    before and after the fixes, its statistics and its <DUP> spans.  The snp
    and small lists stay in pg_region_fixes' packed form (`fixes`, `text`)
    and become Fix objects only where reassembly or the VCF asks for them."""

    def __init__(self, contig, start, stop, bases, stats=None):
        self.contig, self.start, self.stop, self.bases, self.stats = contig, start, stop, bases, stats
        self.big = []           # local reassemblies and gap fills
        self.dupes = []
        self.bases_snp = None   # the bases after the SNP fixes alone
        self.orig = None
        self.fixes = np.zeros(0, _abi.fix_dtype())
        self.text = b""
        self._lists = None

    def _decoded(self):
        if self._lists is None:
            snp, small, t = [], [], self.text
            for locus, lst, wo, wl, po, pl in self.fixes.tolist():
                (snp if lst == 0 else small).append(Fix(locus, t[wo:wo + wl].decode(), t[po:po + pl].decode()))
            self._lists = (snp, small)
        return self._lists

    @property
    def snp(self):
        return self._decoded()[0]

    @property
    def small(self):
        return self._decoded()[1]

    def all_fixes(self):
        return fix_fix_list(self.snp + self.small + self.big)

    def packed_fixes(self):
        """snpFixList ++ smallFixList ++ bigFixList as (pg_fix array, text)."""
        if not self.big:
            return self.fixes, self.text
        text = bytearray(self.text)
        big = np.zeros(len(self.big), _abi.fix_dtype())
        for k, f in enumerate(self.big):
            was, patch = f.was.encode(), f.patch.encode()
            big[k] = (f.locus, 2, len(text), len(was), len(text) + len(was), len(patch))
            text += was + patch
        return np.concatenate([self.fixes, big]), bytes(text)


def _region_outputs(engine, r, region, ref, opts, params, changes, chars, dupes=()):
    """The region's changes (pg_fetch_changes: pass-1 changes in locus order,
    insertion characters) -> fix lists and fixed bases (pg_region_fixes); its
    duplication events (pg_find_duplications) -> where its <DUP> records go."""
    c, s, e, _, _ = region
    st = engine.stats(r)
    orig = bytes(ref[s - 1:e])
    excluded = None
    if opts.longread and opts.nanopore is not None and opts.longread_only:
        excluded = _exclude_motifs(orig, s, e, opts.nanopore)
    fixes, text, bases_snp, bases = region_fixes(changes, chars, ref, s, e, fix_snps=opts.fix_snps,
                                                 fix_indels=opts.fix_indels, iupac=opts.iupac,
                                                 long_read=bool(opts.longread), excluded=excluded)
    res = RegionResult(c, s, e, bytearray(bases), stats=st)
    res.fixes, res.text = fixes, text
    res.bases_snp = bytearray(bases_snp)
    res.orig = orig
    res.dupes = list(dupes)
    return res


def _first_lines(engine, r, size):
    """Line of the first VCF record of each position of region r: one record per
    position, plus one after an indel call at i > 0 outside a deletion."""
    call = np.empty(size, np.uint32)
    o = _abi.pg_region_out()
    o.call = call.ctypes.data
    engine._check(engine.L.pg_fetch_region(engine.h, r, C.byref(o)))
    extra = ((call & (_abi.PG_CALL_INS | _abi.PG_CALL_DEL)) != 0) & ((call & _abi.PG_CALL_DELETED) == 0)
    extra[0] = False
    return np.concatenate([[0], np.cumsum(1 + extra.astype(np.int64))])


def _reassemble(engine, regions, results, contigs, reads, params, opts):
    """The gaps and local steps of identifyAndFixIssues (S/GenomeRegion.scala:
    382-413) for every region: one K-mer tally for all windows, then the walks.
    The insert statistics a region's GapFiller sees are those of the scan and
    of the regions processed up to it, as Pilon processes chunks in order."""
    import time
    stats = getattr(opts, "stats", None)  # a dict receives the step times and counts when given
    t0 = time.perf_counter()
    bam = reassembly.BamState(reads, params, len(contigs), strays=opts.strays)
    t1 = time.perf_counter()
    breaks = engine.find_breaks() if opts.fix_local else {}
    jobs, lists, owner = [], [], []
    for r, (reg, res) in enumerate(zip(regions, results)):
        bam.add_region(res.stats)
        c, s, e = reg[0], reg[1], reg[2]
        todo = []
        if opts.fix_gaps:
            todo += [(g, True) for g in reassembly.gaps(contigs[c], s, e)]
        if opts.fix_local:
            todo += [(b, False) for b in breaks.get(r, [])]
        if not todo:
            continue
        radius = bam.break_radius(opts.K)
        bases = np.frombuffer(bytes(res.bases_snp), np.uint8).copy()
        orig = np.frombuffer(res.orig, np.uint8).copy()
        for (bs, be), is_gap in todo:
            lists.append(bam.recruit(c, bs, be))
            jobs.append(dict(window=len(lists) - 1, is_gap=is_gap, region_start=s, region_stop=e, break_start=bs,
                             break_stop=be, break_radius=radius, bases=bases, orig=orig,
                             fix_breaks=opts.fix_breaks, gap_margin=opts.gap_margin, min_gap=opts.min_gap))
            owner.append(r)
    t2 = time.perf_counter()
    if not jobs:
        return
    from .engine import reassemble, EngineError
    edges = engine.kmer_tally_reads(lists, opts.K, params)
    t3 = time.perf_counter()
    fixes = reassemble(edges, opts.K, jobs)
    t4 = time.perf_counter()
    if stats is not None:
        stats.update(scan_s=t1 - t0, recruit_s=t2 - t1, tally_s=t3 - t2, walk_s=t4 - t3, windows=len(jobs),
                     reads=int(sum(len(x) for x in lists)), edges=int(edges.size),
                     tally_device_ms=engine.last_tally_stats()[0] if hasattr(engine, "last_tally_stats") else None,
                     fixes=int(sum(1 for f in fixes if f[0] > 0)))
    for j, r, (start, was, patch, status, _loop) in zip(jobs, owner, fixes):
        if status:
            raise EngineError(status, f"region {r}: the reference would throw reassembling "
                                      f"{j['break_start']}-{j['break_stop']}")
        if start > 0 and (j["is_gap"] or max(len(was), len(patch)) > 10):
            results[r].big.append(Fix(start, was, patch))
    for reg, res in zip(regions, results):
        if res.big:
            res.big.reverse()  # prepended (::=) in the reference
            res.bases = fix_issues(res.bases_snp, reg[1], res.small + res.big)


def _exclude_motifs(orig, s, e, nano):
    """GenomeRegion.excludeMotifs (S/GenomeRegion.scala:416-439): homoRun(i) >= 4,
    the run of equal bases from i rightwards inside the region, is the base at i
    equal to the next three; nanoporeExclude(i) is C C x G G around i with all
    five inside the region."""
    b = np.frombuffer(bytes(orig).upper(), np.uint8)
    n = b.size
    ex = np.zeros(n, bool)
    if n >= 4:
        ex[:n - 3] = (b[:-3] == b[1:-2]) & (b[1:-2] == b[2:-1]) & (b[2:-1] == b[3:])
    if nano and n >= 5:
        C, G = ord("C"), ord("G")
        ex[2:n - 2] |= (b[:n - 4] == C) & (b[1:n - 3] == C) & (b[3:n - 1] == G) & (b[4:] == G)
    return ex


VCF_HEADER_TAIL = (
    '##FILTER=<ID=LowCov,Description="Low Coverage of good reads at location">\n'
    '##FILTER=<ID=Amb,Description="Ambiguous evidence in haploid genome">\n'
    '##FILTER=<ID=Del,Description="This base is in a deletion or change event from another record">\n'
    '##INFO=<ID=DP,Number=1,Type=Integer,Description="Valid read depth; some reads may have been filtered">\n'
    '##INFO=<ID=TD,Number=1,Type=Integer,Description="Total read depth including bad pairs">\n'
    '##INFO=<ID=PC,Number=1,Type=Integer,Description="Physical coverage of valid inserts across locus">\n'
    '##INFO=<ID=BQ,Number=1,Type=Integer,Description="Mean base quality at locus">\n'
    '##INFO=<ID=MQ,Number=1,Type=Integer,Description="Mean read mapping quality at locus">\n'
    '##INFO=<ID=QD,Number=1,Type=Integer,Description="Variant confidence/quality by depth">\n'
    '##INFO=<ID=BC,Number=4,Type=Integer,Description="Count of As, Cs, Gs, Ts at locus">\n')
VCF_QE = '##INFO=<ID=QE,Number=4,Type=Integer,Description="Evidence for As, Cs, Gs, Ts weighted by Q & MQ at locus">\n'
VCF_QP = ('##INFO=<ID=QP,Number=4,Type=Integer,Description="Percentage of As, Cs, Gs, Ts weighted by Q & MQ at '
          'locus">\n')
VCF_HEADER_END = (
    '##INFO=<ID=IC,Number=1,Type=Integer,Description="Number of reads with insertion here">\n'
    '##INFO=<ID=DC,Number=1,Type=Integer,Description="Number of reads with deletion here">\n'
    '##INFO=<ID=XC,Number=1,Type=Integer,Description="Number of reads clipped here">\n'
    '##INFO=<ID=AC,Number=A,Type=Integer,Description="Allele count in genotypes, for each ALT allele, in the same '
    'order as listed">\n'
    '##INFO=<ID=AF,Number=A,Type=Float,Description="Fraction of evidence in support of alternate allele(s)">\n'
    '##INFO=<ID=SVTYPE,Number=1,Type=String,Description="Type of structural variant">\n'
    '##INFO=<ID=SVLEN,Number=.,Type=String,Description="Difference in length between REF and ALT alleles">\n'
    '##INFO=<ID=END,Number=1,Type=Integer,Description="End position of the variant described in this record">\n'
    '##INFO=<ID=IMPRECISE,Number=0,Type=Flag,Description="Imprecise change from local reassembly (ALT contains '
    'Ns)">\n'
    '##FORMAT=<ID=GT,Number=1,Type=String,Description="Genotype">\n'
    '##FORMAT=<ID=AD,Number=.,Type=String,Description="Allelic depths for the ref and alt alleles in the order '
    'listed">\n'
    '##FORMAT=<ID=DP,Number=1,Type=String,Description="Approximate read depth; some reads may have been filtered">\n'
    '##ALT=<ID=DUP,Description="Possible segmental duplication">\n'
    '#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT\tSAMPLE\n')


def vcf_header(contigs_with_sizes, opts):
    """Vcf.writeHeader (S/Vcf.scala:28-68)."""
    h = (f"##fileformat=VCFv4.1\n##fileDate={opts.vcf_date}\n##source=\"{opts.vcf_source}\"\n"
         f"##PILON=\"{opts.vcf_args}\"\n##reference={opts.vcf_ref}\n")
    for c, s in contigs_with_sizes:
        h += f"##contig=<ID={c},length={s}>\n"
    return h + VCF_HEADER_TAIL + (VCF_QE if opts.vcf_qe else VCF_QP) + VCF_HEADER_END


def new_name(name):  # S/GenomeFile.scala:137-140
    sep = "_" if "|" not in name else ("" if name.endswith("|") else "|")
    return name + sep + "pilon"


def polish(engine, names, contigs, reads, params, out_prefix, opts=None, batched=True):
    """Runs the engine over every region and writes out_prefix.{fasta,vcf,changes}.
    Returns the per-region results."""
    opts = opts or Options()
    opts.longread_only = bool(opts.longread) and bool(getattr(opts, "no_frags", False))
    lens = [int(c.size) for c in contigs]
    regions = plan_regions(reads, lens, opts.chunk_size, opts.targets, opts.contig_order)
    engine.set_reference(contigs)
    engine.set_reads(reads)
    engine.pileup_regions(regions, params, batched=batched)
    # pass 2 of postProcess and duplicationEvents, on the device (the <DUP> records)
    dups = engine.find_duplications() if opts.vcf else {}
    # the pass-1 changes of all regions at once, ordered by region and locus
    changes, chars = engine.fetch_changes()
    bounds = np.searchsorted(changes["region"], np.arange(len(regions) + 1, dtype=changes["region"].dtype))
    results = [_region_outputs(engine, r, reg, contigs[reg[0]], opts, params, changes[bounds[r]:bounds[r + 1]],
                               chars, dups.get(r, ())) for r, reg in enumerate(regions)]
    if opts.fix_gaps or opts.fix_local:
        _reassemble(engine, regions, results, contigs, reads, params, opts)
    # The output groups of GenomeFile.regions (S/GenomeFile.scala:49-54): a contig
    # with its chunks, or with --targets one group per target (two targets on one
    # contig give two FASTA records, and each restarts the changes offset).
    groups = []
    for r, res in enumerate(results):
        if opts.targets is None and groups and groups[-1][0] == res.contig:
            groups[-1][1].append(r)
        else:
            groups.append((res.contig, [r]))
    if opts.vcf:
        with open(out_prefix + ".vcf", "wb") as vf:
            sizes = [(names[c], sum(results[r].stop - results[r].start + 1 for r in rs)) for c, rs in groups]
            vf.write(vcf_header(sizes, opts).encode())
            for r, res in enumerate(results):
                inserts = _vcf_inserts(engine, r, res, names[res.contig], contigs[res.contig])
                text = engine.format_vcf(r, names[res.contig], opts.diploid, opts.vcf_qe)
                if inserts:
                    text = _splice(text, _first_lines(engine, r, res.stop - res.start + 1), inserts, res.start)
                vf.write(text)
    if opts.changes:
        with open(out_prefix + ".changes", "wb") as cf:
            for c, rs in groups:
                name, nn = names[c], new_name(names[c])
                offset = 0
                for r in rs:
                    res = results[r]
                    fixes, text = res.packed_fixes()
                    cf.write(changes_lines(fixes, text, name, nn, offset))
                    offset += len(res.bases) - (res.stop - res.start + 1)
    if opts.fix_snps or opts.fix_indels or opts.fix_gaps or opts.fix_local:
        with open(out_prefix + ".fasta", "wb") as ff:
            for c, rs in groups:
                seq = b"".join(bytes(results[r].bases) for r in rs)
                ff.write(b">" + new_name(names[c]).encode() + b"\n")
                ff.write(fasta_lines(seq))
    return results


def _vcf_inserts(engine, r, res, name, ref):
    """The records GenomeRegion.writeVcf writes before a position's own
    (S/GenomeRegion.scala:623-643): Vcf.writeDup at a duplication's first
    locus (S/Vcf.scala:194-202), then Vcf.writeFixRecord at the first locus of
    a fix that only local reassembly made (S/Vcf.scala:178-192), whose
    replaced loci are marked deleted on the device first.  A list of (locus,
    line) in writing order."""
    out = [(d[0], (f"{name}\t{d[0] - 1}\t.\t{chr(ref[d[0] - 2]).upper()}\t<DUP>\t.\tPASS\tSVTYPE=DUP;"
                   f"SVLEN={d[1] + 1 - d[0]};END={d[1]};IMPRECISE\tGT\t./.").encode()) for d in res.dupes]
    if res.big:
        small = {(f.locus, f.was, f.patch) for f in res.small}
        big = {(f.locus, f.was, f.patch) for f in res.big}
        for f in res.all_fixes():
            key = (f.locus, f.was, f.patch)
            if key in big and key not in small:
                loc = f.locus - 1
                if loc < res.start:
                    raise IndexError(f"{name}:{f.locus}: the reference's refBase({loc}) is outside the region")
                rb = chr(ref[loc - 1]).upper()
                rs, alt = rb + f.was, rb + f.patch
                svlen = len(alt) - len(rs)
                line = (f"{name}\t{loc}\t.\t{rs}\t{alt}\t.\tPASS\tSVTYPE={'DEL' if svlen < 0 else 'INS'};"
                        f"SVLEN={svlen};END={loc + len(rs) - 1}{';IMPRECISE' if 'N' in f.patch else ''}\tGT\t1/1")
                out.append((f.locus, line.encode()))
                if f.was:
                    engine.mark_deleted(r, f.locus, len(f.was))
    out.sort(key=lambda x: x[0])  # stable: a duplication's record stays before a fix's at the same locus
    return out


def _splice(text, first_line, inserts, start):
    """Inserts the (locus, line) records before the records of their locus."""
    lines = text.split(b"\n")
    out = []
    prev = 0
    for locus, line in inserts:
        k = int(first_line[locus - start])
        out.extend(lines[prev:k])
        out.append(line)
        prev = k
    out.extend(lines[prev:])
    return b"\n".join(out)
