"""Known-answer tests of the CPU oracle, derived by hand from the Scala source.

The reference ships no tests, fixtures or golden vectors and cannot run here
(no JVM), so each expected value below is worked out from the cited Scala
lines.  One case per parity hazard of the hot path:
  H1 deletion left shift adds bases without removing them   S/PileUpRegion.scala:163-183
  H2 a homozygous deletion updates the pileups it covers    S/GenomeRegion.scala:259-264
  H3 a left shift below the region start throws             S/PileUpRegion.scala:155-182
  H4 indels count by their region bounds (pre-shift locus)  S/PileUpRegion.scala:155,166
  long-read indels: mq min 8, homopolymer runs dropped      S/PileUpRegion.scala:120-126,142-183
  nanopore CC?GG motif bases at quality 0 (region index)    S/PileUpRegion.scala:128-134,189
  long reads only: run starts of 4+ bases are not fixed     S/GenomeRegion.scala:326,416-439
  H5 integer rounding (roundDiv, adjMq)                     S/Utils.scala:23-26, S/PileUpRegion.scala:139-142
  H5 BaseCall score, q and highConfidence arithmetic        S/PileUp.scala:132-153
  H6 stable base order on ties                              S/BaseSum.scala:57-60
  indel call thresholds (insertions and deletions)          S/PileUp.scala:182-247
  H7 insert-size statistics per region (FR / RF), cutoff    S/BamFile.scala:161-165,192-202
  a placed unmapped read (alignment end 0): physCov [0,pos)  S/PileUpRegion.scala:62-100
  minDepth: (0.1 * meanCoverage).round max 5                S/GenomeRegion.scala:221-224
  H9 K-mer tally read rules (length, clips, N, minQual)     S/Assembler.scala:55-87
  H10 Java "%.2f" rounding of AF                            S/Vcf.scala:134-152
  AMB fixes: base, IUPAC code, --fix amb, long reads        S/GenomeRegion.scala:265-269,331-340
  changes lines and FASTA after indel fixes, across chunks  S/GenomeRegion.scala:595-657, S/GenomeFile.scala:140-160
  soft-masked (lowercase) reference: raw in indel shifts     S/PileUpRegion.scala:156, S/GenomeRegion.scala:783-787
  VCF records: REF/ALT/GT, filters, BQ/MQ/QD/QP/AF fields  S/Vcf.scala:74-176, S/PileUp.scala:55-71
  H12 output names, FASTA wrapping, changes format          S/GenomeFile.scala:79-82,135-161
"""
import os
import tempfile

import numpy as np
import pytest

from oracle import oracle
from pilon_gb300 import _abi
from pilon_gb300.reads import build_store


def ref_from(seq):
    return np.frombuffer(seq.encode(), np.uint8).copy()


def rand_ref(n, seed=7, avoid_runs=True):
    rng = np.random.Generator(np.random.PCG64(seed))
    s = []
    for _ in range(n):
        while True:
            c = "ACGT"[rng.integers(0, 4)]
            if not avoid_runs or not s or c != s[-1]:
                break
        s.append(c)
    return "".join(s)


def read(pos, cigar, seq, qual=30, mapq=60, flag=0, tlen=0):
    q = None if qual is None else ([qual] * len(seq) if isinstance(qual, int) else qual)
    return dict(pos=pos, cigar=cigar, seq=seq, qual=q, mapq=mapq, flag=flag, tlen=tlen)


def run(ref, records, start=1, stop=None, **pk):
    st = build_store(records)
    stop = len(ref) if stop is None else stop
    return oracle.process_region(st, _abi.default_params(**pk), ref_from(ref), 0, start, stop)


def at(res, locus, start=1):
    i = locus - start
    return dict(count=res.count[4 * i:4 * i + 4].tolist(), qual_sum=res.qual_sum[4 * i:4 * i + 4].tolist(),
                mq=int(res.mq_sum[i]), q=int(res.q_sum[i]), bad=int(res.bad_pair[i]), clips=int(res.clips[i]),
                dels=int(res.deletions[i]), ins=int(res.insertions[i]), pc=int(res.phys_cov[i]),
                isz=int(res.insert_size[i]), call=int(res.call[i]))


def test_single_read_trusted_flank_and_physcov():
    ref = rand_ref(300)
    seq = ref[100:140]                           # 40M at locus 101..140
    res = run(ref, [read(101, [(40, "M")], seq)])
    assert res.status == 0
    # trusted offsets are 10..29 (flank 10): loci 111..130
    assert at(res, 110)["count"] == [0, 0, 0, 0] and at(res, 131)["count"] == [0, 0, 0, 0]
    b = "ACGT".index(ref[110])
    p = at(res, 111)
    assert p["count"][b] == 1 and p["qual_sum"][b] == 30 * 61 and p["mq"] == 61 and p["q"] == 30
    assert res.stats.base_count == 20 and res.stats.read_count == 1
    # unpaired: physical coverage [min(aStart,aEnd), max) = [101, 140): +1 at 101, -1 at 140
    assert at(res, 100)["pc"] == 0 and at(res, 101)["pc"] == 1 and at(res, 139)["pc"] == 1 and at(res, 140)["pc"] == 0
    assert at(res, 120)["isz"] == 39


def test_soft_clips_bad_pairs_and_adjusted_mq():
    ref = rand_ref(300)
    seq = "ACGTA" + ref[99:129]                  # 5S30M at 100
    res = run(ref, [read(100, [(5, "S"), (30, "M")], seq)])
    # clipStart = locus - len = 95 (clip at read start), clipEnd = 99
    assert at(res, 95)["clips"] == 1 and at(res, 99)["clips"] == 1 and at(res, 97)["clips"] == 0
    assert [at(res, l)["bad"] for l in range(94, 101)] == [0, 1, 1, 1, 1, 1, 0]
    # adjMq = roundDiv(60 * (35 - 5), 35) = (1800 + 17) / 35 = 51 -> mq + 1 = 52
    assert at(res, 110)["mq"] == 52
    # trailing clip: clipStart = locus (130), clipEnd = 134
    seq2 = ref[99:129] + "TTTTT"
    res2 = run(ref, [read(100, [(30, "M"), (5, "S")], seq2)])
    assert at(res2, 130)["clips"] == 1 and at(res2, 134)["clips"] == 1
    assert [at(res2, l)["bad"] for l in range(129, 136)] == [0, 1, 1, 1, 1, 1, 0]


def test_single_base_clip_counts_twice():
    ref = rand_ref(200)
    res = run(ref, [read(50, [(1, "S"), (30, "M")], "A" + ref[49:79])])
    # clipStart == clipEnd == 49: both increments land on the same pileup
    assert at(res, 49)["clips"] == 2


def test_H1_deletion_left_shift_double_counts():
    # loci 146..149 = "CAAA", 150..153 "AAGT"... build: ...C A A A A G...
    ref = list(rand_ref(300))
    ref[148] = "C"                                # locus 149
    for l in (150, 151, 152, 153):
        ref[l - 1] = "A"
    ref[153] = "G"                                # locus 154
    ref = "".join(ref)
    # read: 30M at 123..152, 1D at 153, 30M at 154..183
    seq = ref[122:152] + ref[153:183]
    res = run(ref, [read(123, [(30, "M"), (1, "D"), (30, "M")], seq)])
    # the deletion slides from 153 to 150 (loci 149 'C' != 150 'A' stops it);
    # each step adds the read base at rloc to locus dloc + 1 = 153, 152, 151
    cA = lambda l: at(res, l)["count"][0]
    assert cA(150) == 1 and cA(151) == 2 and cA(152) == 2 and cA(153) == 1
    assert at(res, 150)["dels"] == 1 and at(res, 153)["dels"] == 0
    # baseCount: 20 + 20 trusted M bases? offsets 10..49 of a 60-base read = 40, plus 3 shifted adds
    assert res.stats.base_count == 43


def test_insertion_left_shift_rotates():
    ref = list(rand_ref(400))
    for k, c in zip(range(300, 306), "TACACG"):  # loci 300..305
        ref[k - 1] = c
    ref[298] = "G"
    ref = "".join(ref)
    # 30M ending at 304, 2I "AC", 30M from 305
    seq = ref[274:304] + "AC" + ref[304:334]
    res = run(ref, [read(275, [(30, "M"), (2, "I"), (30, "M")], seq)] * 6)
    # iloc slides 305 -> 301 over four steps; the string rotates AC->CA->AC->CA->AC
    assert at(res, 301)["ins"] == 6 and at(res, 305)["ins"] == 0
    i = 301 - 1
    assert res.call[i] & _abi.PG_CALL_INS and res.insertion(i) == "AC"


def test_H2_homozygous_deletion_updates_covered_pileups():
    ref = rand_ref(400, seed=11)
    recs = []
    for k in range(8):
        p = 150 + 2 * k
        d = 200                                   # delete loci 200..202
        seq = ref[p - 1:d - 1] + ref[d + 2:d + 2 + 40]
        recs.append(read(p, [(d - p, "M"), (3, "D"), (40, "M")], seq))
    res = run(ref, recs)
    i = 200 - 1
    assert at(res, 200)["dels"] == 8
    assert (res.call[i] >> 9) & 7 == _abi.PG_CHANGE_DEL and res.indel_len[i] == 3
    # pass 1 marks 201 and 202 deleted and adds the 8 deletions to them
    for l in (201, 202):
        assert at(res, l)["dels"] == 8 and at(res, l)["call"] & _abi.PG_CALL_DELETED
        assert (at(res, l)["call"] >> 9) & 7 == 0
    assert at(res, 203)["dels"] == 0


def test_H3_left_shift_below_region_start_throws():
    ref = list(rand_ref(300))
    for l in range(95, 106):
        ref[l - 1] = "A"
    ref = "".join(ref)
    seq = ref[79:101] + ref[102:130]             # 22M at 80..101, 1D at 102, 28M at 103..130
    res = run(ref, [read(80, [(22, "M"), (1, "D"), (28, "M")], seq)], start=101, stop=300)
    assert res.status == _abi.PG_ERR_INDEX
    # the same read on a region starting at 1 is fine (shift stops at 95)
    res = run(ref, [read(80, [(22, "M"), (1, "D"), (28, "M")], seq)])
    assert res.status == 0 and at(res, 95)["dels"] == 1


def test_H6_stable_order_on_ties():
    ref = rand_ref(200)
    l = 100
    base = ref[l - 1]
    alts = [c for c in "ACGT" if c != base]
    a, b = alts[0], alts[1]                       # a < b in ACGT order
    recs = []
    for c in (a, b):
        s = list(ref[79:129])
        s[l - 80] = c
        recs.append(read(80, [(50, "M")], "".join(s)))
    res = run(ref, recs)
    f = int(res.call[l - 1])
    assert "ACGT"[f & 3] == a and "ACGT"[(f >> 2) & 3] == b
    assert not f & _abi.PG_CALL_HOMO


def test_validate_read_flags():
    ref = rand_ref(300)
    seq = ref[99:139]
    recs = [read(100, [(40, "M")], seq, flag=0x400), read(100, [(40, "M")], seq, flag=0x100),
            read(100, [(40, "M")], seq, flag=0x200), read(100, [(40, "M")], seq, flag=0x800)]
    res = run(ref, recs)
    assert res.stats.read_count == 1               # only the supplementary read is kept
    res = run(ref, recs, duplicates=1, nonpf=1)
    assert res.stats.read_count == 3               # secondary reads are always dropped


def test_paired_read_before_region_carries_physcov():
    ref = rand_ref(400)
    seq = ref[49:99]
    # proper pair, leftmost mate at 50, TLEN 300 -> insert [50, 350); region starts at 101
    res = run(ref, [read(50, [(50, "M")], seq, flag=0x1 | 0x2 | 0x20 | 0x40, tlen=300)], start=101, stop=400)
    assert res.stats.phys_cov_start == 1 and res.stats.insert_size_start == 300
    assert at(res, 101, start=101)["pc"] == 1 and at(res, 349, start=101)["pc"] == 1
    assert at(res, 350, start=101)["pc"] == 0 and at(res, 200, start=101)["isz"] == 300


def test_invalid_pair_goes_to_bad_pairs():
    ref = rand_ref(300)
    seq = ref[99:139]
    res = run(ref, [read(100, [(40, "M")], seq, flag=0x1 | 0x40, tlen=100)])  # paired, not proper
    assert at(res, 120)["bad"] == 1 and at(res, 120)["count"] == [0, 0, 0, 0]
    assert res.stats.base_count == 0


def test_missing_qualities_use_default():
    ref = rand_ref(300)
    res = run(ref, [read(100, [(40, "M")], ref[99:139], qual=None)], default_qual=17)
    assert at(res, 120)["q"] == 17


@pytest.mark.parametrize("x,s", [(0.125, "0.13"), (0.375, "0.38"), (0.0, "0.00"), (1.0, "1.00"),
                                 (float(np.float32(1) / np.float32(3)), "0.33"),
                                 (float(np.float32(2) / np.float32(3)), "0.67"), (0.005, "0.01"),
                                 (0.015, "0.02"), (0.994999, "0.99"), (0.995, "1.00"), (0.5, "0.50")])
def test_H10_java_half_up_format(x, s):
    assert oracle.java_format2(x) == s


def test_contig_chunking():
    # GenomeFile.contigRegions: nChunks = ceil(len/max), chunk = ceil(len/nChunks)
    assert oracle.contig_regions(25, 10) == [(1, 9), (10, 18), (19, 25)]
    assert oracle.contig_regions(20, 10) == [(1, 10), (11, 20)]
    from pilon_gb300.regions import contig_regions
    for n, c in [(25, 10), (20, 10), (1, 10), (10_000_001, 10_000_000), (123_456, 7_000)]:
        assert contig_regions(n, c) == oracle.contig_regions(n, c)


def test_H12_fasta_changes_naming():
    ref = rand_ref(2000, seed=3)
    sample = list(ref)
    sample[999] = "ACGT"[("ACGT".index(ref[999]) + 1) % 4]   # SNP at locus 1000
    sample = "".join(sample)
    recs = []
    for p in range(1, 1900, 5):
        recs.append(read(p, [(100, "M")], sample[p - 1:p + 99]))
    st = build_store(recs)
    with tempfile.TemporaryDirectory() as d:
        for name, out in [("chr1", "chr1_pilon"), ("gi|123|", "gi|123|pilon"), ("gi|123", "gi|123|pilon")]:
            pre = os.path.join(d, "o")
            assert oracle.polish(st, _abi.default_params(), [name], [ref_from(ref)], pre) == 0
            fa = open(pre + ".fasta").read().splitlines()
            assert fa[0] == ">" + out
            assert all(len(l) == 80 for l in fa[1:-1]) and len(fa[-1]) == 2000 - 80 * (len(fa) - 2)
            assert "".join(fa[1:])[999] == sample[999]
            ch = open(pre + ".changes").read().splitlines()
            assert ch == [f"{name}:1000 {out}:1000 {ref[999]} {sample[999]}"]
            vcf = open(pre + ".vcf").read().splitlines()
            body = [l for l in vcf if not l.startswith("#")]
            assert len(body) == 2000
            f = body[999].split("\t")
            assert f[1] == "1000" and f[3] == ref[999] and f[4] == sample[999] and f[9] == "1/1"


def test_kmer_tally_hand_case():
    # five identical reads "ACGTTACG" (L=8), K=3: forward K-mers ACG->T, CGT->T, GTT->A, TTA->C, TAC->G
    # reverse complement "CGTAACGT": CGT->A, GTA->A, TAA->C, AAC->G, ACG->T
    recs = [read(10, [(8, "M")], "ACGTTACG", qual=30, mapq=20)] * 5
    st = build_store(recs)
    e = oracle.kmer_tally(st, _abi.default_params(), [(0, 5)], 3, min_depth=5)
    nib = {"A": 1, "C": 2, "G": 4, "T": 8}
    def key(k):
        v = 0
        for j, c in enumerate(k):
            v |= nib[c] << (60 - 4 * j)
        return v
    got = {(int(x["key_hi"]), int(x["next"]), int(x["alt"]), int(x["depth"])) for x in e}
    # CGT: 5 x T (forward) and 5 x A (reverse): tie on qual sums -> base A (lower index), het -> alt T
    exp = {(key("ACG"), 3, -1, 10), (key("CGT"), 0, 3, 10), (key("GTT"), 0, -1, 5), (key("TTA"), 1, -1, 5),
           (key("TAC"), 2, -1, 5), (key("GTA"), 0, -1, 5), (key("TAA"), 1, -1, 5), (key("AAC"), 2, -1, 5)}
    assert got == exp



def test_kmer_tally_depth_cut():
    """buildGraph keeps K-mers with depth >= minDepth (S/Assembler.scala:138):
    four copies of the read above give depth 8 to ACG and CGT (both strands) and
    4 to the rest, so only those two have edges; CGT ties 4 T against 4 A."""
    st = build_store([read(10, [(8, "M")], "ACGTTACG", qual=30, mapq=20)] * 4)
    e = oracle.kmer_tally(st, _abi.default_params(), [(0, 4)], 3, min_depth=5)
    got = {(int(x["next"]), int(x["alt"]), int(x["depth"])) for x in e}
    assert len(e) == 2 and got == {(3, -1, 8), (0, 3, 8)}

def test_summary_regions_merge_rule():
    """GenomeRegion.summaryRegions closes a run at the first untested position
    more than slop past the last tested one (S/GenomeRegion.scala:748-757):
    tested positions slop + 1 apart stay in one run, slop + 2 apart split."""
    from tests.breaks_host import summary_regions

    def scala(test, start, stop, slop):  # the loop as written in the reference
        regs, first, last = [], -1, -1
        for i in range(test.size):
            if test[i]:
                last = i
                if first < 0:
                    first = i
            elif last >= 0 and i > last + slop:
                regs.append((start + first, start + last))
                first = last = -1
        if last >= 0:
            regs.append((start + first, start + last))
        return [r for r in regs if not (r[0] - start < 100 or stop - r[1] < 100)]

    n = 2000
    for gap in (199, 200, 201, 202, 203):
        t = np.zeros(n, bool)
        t[[500, 500 + gap, 1500]] = True
        got = summary_regions(t, 1, n, 200)
        assert got == scala(t, 1, n, 200), gap
    assert summary_regions(np.isin(np.arange(n), [500, 701]), 1, n, 200) == [(501, 702)]
    assert summary_regions(np.isin(np.arange(n), [500, 702]), 1, n, 200) == [(501, 501), (703, 703)]
    rng = np.random.Generator(np.random.PCG64(7))
    for _ in range(50):
        t = rng.random(n) < 0.004
        assert summary_regions(t, 1, n, 100) == scala(t, 1, n, 100)


def _ins_case(n_ins, n_plain, ins="CA"):
    """Reads over a 100-bp reference: n_ins with 20M 2I 20M at 31 (the insertion
    attaches at 51, the position after the first 20 aligned bases; the base
    before it is not the insertion's last character, so it does not shift) and
    n_plain 40M reads at 31.  Quality 30, mapq 60 everywhere."""
    ref = list(rand_ref(100, seed=3))
    ref[49] = "G"  # position 50, before the insertion: not 'A'
    ref = "".join(ref)
    recs = [read(31, [(20, "M"), (len(ins), "I"), (20, "M")], ref[30:50] + ins + ref[50:70]) for _ in range(n_ins)]
    recs += [read(31, [(40, "M")], ref[30:70]) for _ in range(n_plain)]
    return ref, run(ref, recs)


def _het_reads(ref):
    """10 reads 40M at 31 over `ref`: 6 with A at quality 30 and 4 with C at
    quality 20 at locus 50, mapq 60."""
    recs = []
    for k in range(10):
        seq = list(ref[30:70])
        seq[19] = "A" if k < 6 else "C"
        recs.append(read(31, [(40, "M")], "".join(seq), qual=30 if k < 6 else 20))
    return recs


def test_base_call_het_score_and_amb():
    """BaseCall (S/PileUp.scala:132-153) at one position: 6 reads with A at
    quality 30 and 4 with C at quality 20, mapq 60 (mq + 1 = 61).
      qualSum A = 6*30*61 = 10980, C = 4*20*61 = 4880, total 15860, n = 10, mqSum = 610
      homoScore = 10980 - 4880 = 6100; half = 7930;
      heteroScore = 15860 - |7930 - 10980| - |7930 - 4880| = 9760 -> not homozygous
      score = |6100 - 9760| * 10 / 610 = 60, q = 6 (not high confidence)
    The reference base is G: base A != G, score > 0, het and altBase C != G,
    so pass 1 records an ambiguous change (S/GenomeRegion.scala:265-269)."""
    ref = list(rand_ref(100, seed=5))
    ref[49] = "G"
    ref = "".join(ref)
    recs = _het_reads(ref)
    res = run(ref, recs)
    p = at(res, 50)
    assert p["count"] == [6, 4, 0, 0] and p["qual_sum"] == [10980, 4880, 0, 0]
    assert p["mq"] == 610 and p["q"] == 6 * 30 + 4 * 20
    assert int(res.score[49]) == 60
    f = p["call"]
    assert f & 3 == 0 and (f >> 2) & 3 == 1  # base A, alt C
    assert f & _abi.PG_CALL_HAS_BASE and not f & _abi.PG_CALL_HOMO and f & _abi.PG_CALL_HOMO_INDEL
    assert (f >> 9) & 7 == _abi.PG_CHANGE_AMB and not f & _abi.PG_CALL_CONFIRMED
    assert res.stats.min_depth == 5  # 200 trusted bases / 100 positions = 2 -> (0.2).round max 5


@pytest.mark.parametrize("n_ins,n_plain,homo", [(8, 2, True), (5, 5, False), (13, 7, False), (14, 6, True)])
def test_insertion_call_thresholds(n_ins, n_plain, homo):
    """hetIndelCall (S/PileUp.scala:209-247) for "CA" at position 51:
      insPct = max(pct(insQual, mqSum), pct(insertions, count)); insQual = 61 per
      insertion, mqSum = 61 per read (an insertion adds none), count = all reads
      middle = max(45 - 2, 10) = 43, low = 21, high = 2*43 - 21 = 65
    8 of 10 -> 80 > 65: homozygous, an INS change in pass 1;  5 of 10 -> 50: het;
    13 of 20 -> pct(793, 1220) = 65, not above high: het;  14 of 20 -> 70: homozygous."""
    ref, res = _ins_case(n_ins, n_plain)
    p = at(res, 51)
    n = n_ins + n_plain
    assert p["ins"] == n_ins and p["mq"] == 61 * n
    f = p["call"]
    assert f & _abi.PG_CALL_INS and int(res.indel_len[50]) == 2 and res.insertion(50) == "CA"
    assert bool(f & _abi.PG_CALL_HOMO_INDEL) == homo
    assert (f >> 9) & 7 == (_abi.PG_CHANGE_INS if homo else _abi.PG_CHANGE_NONE)
    # homozygous reference base: score = total * n / mqSum = (n * 30 * 61) * n / (61 n) = 30 n
    assert int(res.score[50]) == 30 * n


def test_insertion_gate_needs_three():
    """insertCall needs insertions > 2 (S/PileUp.scala:182-185): 2 of 5 reads
    (pct 40, which would be het) give no call."""
    ref, res = _ins_case(2, 3)
    f = at(res, 51)["call"]
    assert not f & _abi.PG_CALL_INS and (f >> 9) & 7 == _abi.PG_CHANGE_NONE


@pytest.mark.parametrize("n_reads,mean,min_depth", [(270, 54, 5), (275, 55, 6), (325, 65, 7), (370, 74, 7),
                                                   (375, 75, 8)])
def test_min_depth_rounds_half_up(n_reads, mean, min_depth):
    """minDepth = (0.1 * meanCoverage).round max 5 (S/GenomeRegion.scala:221-224),
    meanCoverage = roundDiv(baseCount, size): 40M reads each add 20 trusted bases
    to a 100-bp region; 5.5 rounds to 6 and 6.5 to 7 (half up)."""
    ref = rand_ref(100, seed=9)
    recs = [read(1 + (k % 61), [(40, "M")], ref[k % 61:k % 61 + 40]) for k in range(n_reads)]
    recs.sort(key=lambda r: r["pos"])
    res = run(ref, recs)
    assert res.stats.base_count == 20 * n_reads and (20 * n_reads + 50) // 100 == mean
    assert res.stats.min_depth == min_depth


def test_min_depth_option_at_least_one_is_a_count():
    ref = rand_ref(100, seed=9)
    recs = [read(1 + (k % 61), [(40, "M")], ref[k % 61:k % 61 + 40]) for k in range(300)]
    recs.sort(key=lambda r: r["pos"])
    assert run(ref, recs, min_depth=12.0).stats.min_depth == 12


@pytest.mark.parametrize("md,want", [(12.9, 12), (1e10, 2 ** 31 - 1), (float("inf"), 2 ** 31 - 1),
                                     (float("nan"), 5), (float("-inf"), 5), (-3.0, 5)])
def test_min_depth_option_java_conversions(md, want):
    """minDepth (S/GenomeRegion.scala:221-224) with Java's conversions:
    minDepth >= 1 takes Double.toInt (truncates; saturates at Int.MaxValue);
    otherwise Math.round (NaN -> 0, -inf -> Long.MinValue) then Long.toInt (low
    32 bits: 0) and max 5."""
    ref = rand_ref(100, seed=9)
    recs = [read(1 + (k % 61), [(40, "M")], ref[k % 61:k % 61 + 40]) for k in range(300)]
    recs.sort(key=lambda r: r["pos"])
    assert run(ref, recs, min_depth=md).stats.min_depth == want


def test_kmer_tally_read_rules():
    """Assembler.addRead/addToPileups (S/Assembler.scala:55-87), K = 4, five copies of each read:
      a read of length K adds nothing (length > K is required);
      getReadString includes soft-clipped bases (2S3M "TTCCA": TTCC -> A);
      K-mers holding N are kept (ANGT -> C; its reverse complement GACN -> T);
      a next base that is not A/C/G/T adds nothing (CCCA -> N), but NTGG -> G does;
      a next base below minQual adds nothing (minQual 10: GATC -> G at quality 5),
      while the reverse strand reads the reversed qualities (CGAT -> C at quality 30)."""
    recs = []
    for seq, cig, q in [("ACGTA", [(5, "M")], 30), ("ACGT", [(4, "M")], 30), ("TTCCA", [(2, "S"), (3, "M")], 30),
                        ("ANGTC", [(5, "M")], 30), ("CCCAN", [(5, "M")], 30), ("GATCG", [(5, "M")], [30, 30, 30, 30, 5])]:
        recs += [read(10, cig, seq, qual=q, mapq=20)] * 5
    st = build_store(recs)
    e = oracle.kmer_tally(st, _abi.default_params(min_qual=10), [(0, len(recs))], 4, min_depth=5)
    nib = {"A": 1, "C": 2, "G": 4, "T": 8, "N": 15}

    def key(k):
        v = 0
        for j, c in enumerate(k):
            v |= nib[c] << (60 - 4 * j)
        return v
    got = {(int(x["key_hi"]), int(x["next"]), int(x["alt"]), int(x["depth"])) for x in e}
    idx = {"A": 0, "C": 1, "G": 2, "T": 3}
    exp = {(key(k), idx[b], -1, 5) for k, b in [("ACGT", "A"), ("TACG", "T"), ("TTCC", "A"), ("TGGA", "A"),
                                               ("ANGT", "C"), ("GACN", "T"), ("NTGG", "G"), ("CGAT", "C")]}
    assert got == exp


@pytest.mark.parametrize("n_del,n_plain,homo", [(8, 2, True), (5, 5, False), (13, 7, False), (14, 6, True)])
def test_deletion_call_thresholds(n_del, n_plain, homo):
    """deletionCall and hetIndelCall (S/PileUp.scala:187-247) for a 2-bp deletion
    of loci 51-52 (20M 2D 20M at 31; the base before it differs from its last
    base, so it does not shift).  addDeletion adds mq + 1 to mqSum
    (S/PileUp.scala:107-114), so delPct = max(pct(61 d, 61 n), pct(d, n)) = pct(d, n)
    with n = all reads; len 2: low 21, high 65.  A homozygous call is a DEL change
    and marks locus 52 deleted, adding the deletions to it (S/GenomeRegion.scala:259-264).
    The score comes from the plain reads' bases: 30 * 61 * p * p / (61 n) with p plain reads."""
    ref = list(rand_ref(100, seed=4))
    ref[49], ref[51] = "C", "G"  # loci 50 and 52 differ
    ref = "".join(ref)
    recs = [read(31, [(20, "M"), (2, "D"), (20, "M")], ref[30:50] + ref[52:72]) for _ in range(n_del)]
    recs += [read(31, [(40, "M")], ref[30:70]) for _ in range(n_plain)]
    res = run(ref, recs)
    n = n_del + n_plain
    p = at(res, 51)
    assert p["dels"] == n_del and p["mq"] == 61 * n and p["count"][("ACGT".index(ref[50]))] == n_plain
    f = p["call"]
    assert f & _abi.PG_CALL_DEL and int(res.indel_len[50]) == 2
    assert bool(f & _abi.PG_CALL_HOMO_INDEL) == homo
    assert (f >> 9) & 7 == (_abi.PG_CHANGE_DEL if homo else _abi.PG_CHANGE_NONE)
    assert int(res.score[50]) == 30 * 61 * n_plain * n_plain // (61 * n)
    q52 = at(res, 52)
    assert bool(q52["call"] & _abi.PG_CALL_DELETED) == homo and q52["dels"] == (n_del if homo else 0)


def test_insert_size_statistics():
    """BamFile.addInsert (S/BamFile.scala:194-202) with the size physCovIncr
    returns (S/PileUpRegion.scala:62-88): FR when (size > 0) xor reverse strand,
    else RF; 0 (not added) for invalid reads and pairs with TLEN <= 0; unpaired
    reads count too (end - start of the alignment).
      unpaired forward 40M at 101: 39 -> FR     unpaired reverse 40M at 150: 39 -> RF
      proper pair, forward, TLEN 300 -> FR      proper pair, reverse, TLEN -300 -> none
      proper pair, reverse, TLEN 250 -> RF      improper pair, TLEN 200 -> none (invalid)"""
    ref = rand_ref(600, seed=2)
    P = 0x1 | 0x2
    recs = [read(101, [(40, "M")], ref[100:140]),
            read(150, [(40, "M")], ref[149:189], flag=0x10),
            read(160, [(40, "M")], ref[159:199], flag=P | 0x20, tlen=300),
            read(170, [(40, "M")], ref[169:209], flag=P | 0x10, tlen=-300),
            read(180, [(40, "M")], ref[179:219], flag=P | 0x10, tlen=250),
            read(190, [(40, "M")], ref[189:229], flag=0x1, tlen=200)]
    st = run(ref, recs).stats
    assert (st.fr_count, st.fr_sum, st.fr_sumsq) == (2, 39 + 300, 39 * 39 + 300 * 300)
    assert (st.rf_count, st.rf_sum, st.rf_sumsq) == (2, 39 + 250, 39 * 39 + 250 * 250)
    assert st.read_count == 6


def _wrap32(x):
    return (x + 2 ** 31) % 2 ** 32 - 2 ** 31


@pytest.mark.parametrize("bam_type,tlen,counted", [(_abi.PG_BAM_FRAGS, 2499, True), (_abi.PG_BAM_FRAGS, 2500, False),
                                                   (_abi.PG_BAM_JUMPS, 2500, True),
                                                   (_abi.PG_BAM_JUMPS, 49999, True),
                                                   (_abi.PG_BAM_JUMPS, 50000, False)])
def test_insert_size_cutoff_and_int_square(bam_type, tlen, counted):
    """addInsert counts sizes below huge = 5 * maxInsertSizes(bamType): 2,500 for
    frags, 50,000 for jumps (S/BamFile.scala:29, 192-202; the 10x `huge` of
    process only guards a commented-out warning).  InsertSizeStats.add squares
    the size as a Scala Int before widening it (S/BamFile.scala:161-165), so
    49,999^2 = 2,499,900,001 wraps to -1,795,067,295 in sumSq."""
    ref = rand_ref(600, seed=2)
    rec = read(160, [(40, "M")], ref[159:199], flag=0x1 | 0x2 | 0x20, tlen=tlen)
    st = run(ref, [rec], bam_type=bam_type).stats
    want = (1, tlen, _wrap32(tlen * tlen)) if counted else (0, 0, 0)
    assert (st.fr_count, st.fr_sum, st.fr_sumsq) == want
    assert st.rf_count == 0

@pytest.mark.parametrize("hole", [(400, 449), (600, 615), (300, 303)])
def test_possible_breaks_low_coverage_and_dip(hole):
    """possibleBreaks (S/GenomeRegion.scala:659-763) on a 1,000-bp region read by
    40M reads starting at every locus 1..961 except a hole of starts: with no
    clips, bad pairs or N, breakp(i) = coverage < 5 || dip(fragCoverage, i, 100) /
    mean >= 1.5, where coverage = fragCoverage = the trusted bases at i and mean
    is the plain average (S/NormalDistribution.scala:25-28); runs merge with slop
    200 and runs within 100 of the region's ends are dropped.  The expectation
    below restates those lines directly."""
    ref = rand_ref(1000, seed=13)
    starts = [s for s in range(1, 962) if not hole[0] <= s <= hole[1]]
    res = run(ref, [read(s, [(40, "M")], ref[s - 1:s + 39]) for s in starts])
    cov = np.zeros(1000, np.int64)
    for s in starts:
        cov[s - 1 + 10:s - 1 + 30] += 1  # trusted offsets 10..29
    assert np.array_equal(res.count.reshape(-1, 4).sum(1), cov)
    mean = cov.sum() / cov.size
    size = cov.size

    def breakp(i):
        left, right = cov[max(0, i - 100)], cov[min(size - 1, i + 100)]
        return cov[i] < 5 or ((left - cov[i]) + (right - cov[i])) / mean >= 1.5

    regs, first, last = [], -1, -1
    for i in range(size):
        if breakp(i):
            last = i
            first = i if first < 0 else first
        elif last >= 0 and i > last + 200:
            regs.append((1 + first, 1 + last))
            first = last = -1
    if last >= 0:
        regs.append((1 + first, 1 + last))
    want = [r for r in regs if not (r[0] - 1 < 100 or 1000 - r[1] < 100)]
    assert oracle.region_breaks(build_store([read(s, [(40, "M")], ref[s - 1:s + 39]) for s in starts]),
                                _abi.default_params(), ref_from(ref), 0, 1, 1000) == want
    assert len(want) == (1 if hole[1] - hole[0] > 10 else 0)


def test_vcf_records_by_hand():
    """Vcf.writeRecord (S/Vcf.scala:74-176) for three positions of the 6A/4C case
    above (reads 31..70, trusted loci 41..60, reference G at locus 50, no pairs):
    locus 50, het A over C:  not homo and rBase G != A -> (G, A, "0/1", refDP 4880, altDP 10980);
      FILTER Amb (haploid, 0/1; depth 10 >= minDepth 5); QUAL = score 60
      BQ = roundDiv(15860, roundDiv(610 * 10, 10)) = 26; MQ = roundDiv(610 - 10, 10) = 60; QD = q = 6
      QP = toStringPct: (100 * 10980 + 7930) / 15860 = 69, (100 * 4880 + 7930) / 15860 = 31
      PC = 10 (unpaired reads [31, 70)); AC = 1; AF = 10980 / 15860 = 0.692 -> "0.69"
    locus 45, homozygous reference: total 15860, heteroScore = 15860 - 7930 - 7930 = 0,
      score = 15860 * 10 / 610 = 260, q = 26; ALT "." (cBase == rBase), PASS, AC 0, AF 0.00
    locus 5, no reads: base N, homo (0 >= 0), score 0; ALT "."; LowCov (0 < 5); all sums 0."""
    ref = list(rand_ref(100, seed=5))
    ref[49] = "G"
    ref = "".join(ref)
    recs = _het_reads(ref)
    st = build_store(recs)
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "o")
        assert oracle.polish(st, _abi.default_params(), ["chr1"], [ref_from(ref)], pre) == 0
        body = [l for l in open(pre + ".vcf").read().splitlines() if not l.startswith("#")]
    assert len(body) == 100
    info = "DP=10;TD=10;BQ=26;MQ=60;QD=6;BC=6,4,0,0;QP=69,31,0,0;PC=10;IC=0;DC=0;XC=0;AC=1;AF=0.69"
    assert body[49] == "\t".join(["chr1", "50", ".", "G", "A", "60", "Amb", info, "GT", "0/1"])
    r = ref[44]
    bc = ",".join("10" if b == r else "0" for b in "ACGT")
    qp = ",".join("100" if b == r else "0" for b in "ACGT")
    info = f"DP=10;TD=10;BQ=26;MQ=60;QD=26;BC={bc};QP={qp};PC=10;IC=0;DC=0;XC=0;AC=0;AF=0.00"
    assert body[44] == "\t".join(["chr1", "45", ".", r, ".", "260", "PASS", info, "GT", "0/0"])
    info = "DP=0;TD=0;BQ=0;MQ=0;QD=0;BC=0,0,0,0;QP=0,0,0,0;PC=0;IC=0;DC=0;XC=0;AC=0;AF=0.00"
    assert body[4] == "\t".join(["chr1", "5", ".", ref[4], ".", "0", "LowCov", info, "GT", "0/0"])


def _vcf_body(ref, recs, name="chr1"):
    st = build_store(recs)
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "o")
        assert oracle.polish(st, _abi.default_params(), [name], [ref_from(ref)], pre) == 0
        return [l for l in open(pre + ".vcf").read().splitlines() if not l.startswith("#")]


def _counts(base, n):
    return ",".join(str(n) if b == base else "0" for b in "ACGT")


def test_vcf_het_insertion_records():
    """An indel call writes its record at locus - 1 with the base there prefixed,
    then the position's own record without the indel (S/Vcf.scala:90-104, 175).
    5 of 10 reads insert "CA" before locus 51 (the het case of the insertion
    thresholds): insPct = max(pct(305, 610), pct(5, 10)) = 50 -> refDP 50, altDP 50;
    callType 0/1 -> Amb, AC 1, AF 0.50; QUAL = score of the reference base at 51
    = 18300 * 10 / 610 = 300, q 30; IC = 5 at locus 51."""
    ref = list(rand_ref(100, seed=3))
    ref[49] = "G"
    ref = "".join(ref)
    recs = [read(31, [(20, "M"), (2, "I"), (20, "M")], ref[30:50] + "CA" + ref[50:70]) for _ in range(5)]
    recs += [read(31, [(40, "M")], ref[30:70]) for _ in range(5)]
    body = _vcf_body(ref, recs)
    assert len(body) == 101 and body[49].split("\t")[1] == "50"
    r = ref[50]
    info = (f"DP=10;TD=10;BQ=30;MQ=60;QD=30;BC={_counts(r, 10)};QP={_counts(r, 100)};PC=10;IC=5;DC=0;XC=0;"
            "AC=1;AF=0.50")
    assert body[50] == "\t".join(["chr1", "50", ".", "G", "GCA", "300", "Amb", info, "GT", "0/1"])
    info = info.replace("AC=1;AF=0.50", "AC=0;AF=0.00")
    assert body[51] == "\t".join(["chr1", "51", ".", r, ".", "300", "PASS", info, "GT", "0/0"])


def test_vcf_homozygous_deletion_records():
    """8 of 10 reads delete loci 51-52 (the homozygous deletion case).
    Locus 51 gives three things (S/Vcf.scala:81-90, 120-176):
      the deletion record at 50: REF C + deleted bases, ALT C, QUAL ".", 1/1,
        delPct = pct(8, 10) = 80 -> AF 0.80, AC 2, PASS; DP = depth = 2 bases + 8 deletions
        BQ = roundDiv(3660, roundDiv(610 * 2, 10) = 122) = 30, MQ = roundDiv(600, 10) = 60,
        QD = q = score / n = (3660 * 2 / 610 = 12) / 2 = 6
      the embedded record at 51 (embedded = homozygous deletion): filter Del, DP = count = 2,
        QUAL = score 12, 0/0.
    The pass-1 DEL adds the 8 deletions to locus 52 and marks it deleted
    (S/GenomeRegion.scala:259-264), and writeVcf passes deleted(i) as embedded
    (S/GenomeRegion.scala:641): filter Del, DP = count = 2, depth 10, mqSum 122, so
    BQ = roundDiv(3660, roundDiv(122 * 2, 10) = 24) = 153, MQ = roundDiv(122 - 10, 10) = 11,
    score = 3660 * 2 / 122 = 60, q 30, DC 8; its deletion list is empty, so no indel call there."""
    ref = list(rand_ref(100, seed=4))
    ref[49], ref[51] = "C", "G"
    ref = "".join(ref)
    recs = [read(31, [(20, "M"), (2, "D"), (20, "M")], ref[30:50] + ref[52:72]) for _ in range(8)]
    recs += [read(31, [(40, "M")], ref[30:70]) for _ in range(2)]
    body = _vcf_body(ref, recs)
    assert len(body) == 101 and body[49].split("\t")[1] == "50"
    r51 = ref[50]
    info = (f"DP=10;TD=10;BQ=30;MQ=60;QD=6;BC={_counts(r51, 2)};QP={_counts(r51, 100)};PC=10;IC=0;DC=8;XC=0;"
            "AC=2;AF=0.80")
    assert body[50] == "\t".join(["chr1", "50", ".", "C" + ref[50:52], "C", ".", "PASS", info, "GT", "1/1"])
    info = info.replace("DP=10;", "DP=2;").replace("AC=2;AF=0.80", "AC=0;AF=0.00")
    assert body[51] == "\t".join(["chr1", "51", ".", r51, ".", "12", "Del", info, "GT", "0/0"])
    info = (f"DP=2;TD=10;BQ=153;MQ=11;QD=30;BC={_counts('G', 2)};QP={_counts('G', 100)};PC=10;IC=0;DC=8;"
            "XC=0;AC=0;AF=0.00")
    assert body[52] == "\t".join(["chr1", "52", ".", "G", ".", "60", "Del", info, "GT", "0/0"])


def test_changes_and_fasta_after_indel_fixes():
    """A homozygous SNP at 100, an insertion of "CA" before 301 and a deletion
    of 501-502, every read carrying them.  The fix list (S/GenomeRegion.scala:328-349)
    is [(100, r, s), (301, "", "CA"), (501, r501 r502, "")]; writeChanges
    (S/GenomeRegion.scala:645-657) prints old and new regions with
    Region.regionString (S/Region.scala:41: no "-stop" when size < 2, and an empty
    side has size 0) and shifts new loci by the length change so far:
      chr1:100 chr1_pilon:100 r s
      chr1:301 chr1_pilon:301-302 . CA          (delta becomes 2)
      chr1:501-502 chr1_pilon:503 r501r502 .
    fixIssues (S/GenomeRegion.scala:595-621) applies them from the right, giving
    the sample sequence."""
    ref = list(rand_ref(700, seed=11))
    ref[299] = "G" if ref[298] != "G" and ref[300] != "G" else "T"   # locus 300 is not 'A': no left shift
    ref[99] = "C" if ref[99] != "C" else "A"
    while ref[499] == ref[501]:                                      # locus 500 differs from locus 502
        ref[499] = "ACGT"[("ACGT".index(ref[499]) + 1) % 4]
    ref = "".join(ref)
    snp = "ACGT"[("ACGT".index(ref[99]) + 2) % 4]
    assert ref[299] != "A" and ref[298] != ref[299] and ref[499] != ref[501]
    recs, sample = _tile_reads(ref, snps={100: snp}, ins={301: "CA"}, dels={501: 502})
    assert sample == ref[:99] + snp + ref[100:300] + "CA" + ref[300:500] + ref[502:]
    st = build_store(recs)
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "o")
        assert oracle.polish(st, _abi.default_params(), ["chr1"], [ref_from(ref)], pre) == 0
        ch = open(pre + ".changes").read().splitlines()
        fa = "".join(open(pre + ".fasta").read().splitlines()[1:])
    assert ch == [f"chr1:100 chr1_pilon:100 {ref[99]} {snp}", "chr1:301 chr1_pilon:301-302 . CA",
                  f"chr1:501-502 chr1_pilon:503 {ref[500:502]} ."]
    assert fa == sample


@pytest.mark.parametrize("ref_base,pk,iupac,fixed", [("G", {}, False, "A"), ("G", {}, True, "M"), ("C", {}, False, None),
                                                      ("C", {"fix_amb": 1}, False, "A"),
                                                      ("G", {"long_read": 1}, False, None)])
def test_ambiguous_fix_options(ref_base, pk, iupac, fixed):
    """The 6A/4C position (base A, alt C) under the AMB options:
    pass 1 adds an AMB change when fixamb or altBase != ref (S/GenomeRegion.scala:265-269);
    identifyAndFixIssues fixes it to the base, or to the IUPAC code of base and
    alt (A|C = M) with --iupac, and not at all with long reads
    (S/GenomeRegion.scala:331-340, S/Bases.scala:85-88).
      ref G: alt C != G -> change; fix "A", or "M" with iupac; none with long reads
      ref C: alt C == ref -> change only with fixamb."""
    ref = list(rand_ref(100, seed=5))
    ref[49] = ref_base
    ref = "".join(ref)
    recs = _het_reads(ref)
    st = build_store(recs)
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "o")
        assert oracle.polish(st, _abi.default_params(**pk), ["chr1"], [ref_from(ref)], pre, iupac=iupac) == 0
        ch = open(pre + ".changes").read().splitlines()
        fa = "".join(open(pre + ".fasta").read().splitlines()[1:])
    if fixed is None:
        assert ch == [] and fa == ref
    else:
        assert ch == [f"chr1:50 chr1_pilon:50 {ref_base} {fixed}"] and fa == ref[:49] + fixed + ref[50:]


@pytest.mark.parametrize("diploid,filt", [(False, "Amb"), (True, "PASS")])
def test_vcf_diploid_filter(diploid, filt):
    """--diploid drops the Amb filter of 0/1 records (S/Vcf.scala:122-123)."""
    ref = list(rand_ref(100, seed=5))
    ref[49] = "G"
    ref = "".join(ref)
    recs = _het_reads(ref)
    st = build_store(recs)
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "o")
        assert oracle.polish(st, _abi.default_params(), ["chr1"], [ref_from(ref)], pre, diploid=diploid) == 0
        body = [l for l in open(pre + ".vcf").read().splitlines() if not l.startswith("#")]
    f = body[49].split("\t")
    assert f[4] == "A" and f[6] == filt and f[9] == "0/1"


def _long_read_ref(ins_run, del_run):
    """120 bp: locus 49 'A', then a C run of ins_run bases from locus 50 and 'T';
    locus 79 'G', then a T run of del_run bases from locus 80 and 'A'."""
    ref = list(rand_ref(120, seed=21))
    ref[48] = "A"
    ref[49:49 + ins_run] = "C" * ins_run
    ref[49 + ins_run] = "T"
    ref[78] = "G"
    ref[79:79 + del_run] = "T" * del_run
    ref[79 + del_run] = "A"
    return "".join(ref)


@pytest.mark.parametrize("long_read", [_abi.PG_NOT_LONG_READ, _abi.PG_NANOPORE, _abi.PG_PACBIO])
@pytest.mark.parametrize("ins_run,del_run", [(4, 3), (5, 4)])
def test_long_read_indels_next_to_homopolymers(long_read, ins_run, del_run):
    """Long-read indel rules of addRead (S/PileUpRegion.scala:120-126, 142, 150-183):
    indelMq = adjMq min 8, and an indel is dropped when homoRun >= 4.
    homoRun takes a 0-based index into the contig: for an insertion it is given
    the 1-based locus iloc, so it measures the run from locus iloc + 1; for a
    deletion it is given index(dloc) = dloc - start, which in a region starting at
    1 is the run from locus dloc.
      "G" inserted before locus 50, C run from 50 of ins_run: homoRun = ins_run - 1
        (3: kept, 4: dropped); locus 49 'A' != 'G', so no left shift
      locus 80 deleted, T run from 80 of del_run: homoRun = del_run (3 kept, 4 dropped);
        locus 79 'G' != locus 80 'T', so no left shift; no CC?GG motif around it
    Five reads each, mapq 60: short reads add 61 per indel, long reads 9."""
    ref = _long_read_ref(ins_run, del_run)
    recs = [read(30, [(20, "M"), (1, "I"), (20, "M")], ref[29:49] + "G" + ref[49:69]) for _ in range(5)]
    recs += [read(60, [(20, "M"), (1, "D"), (20, "M")], ref[59:79] + ref[80:100]) for _ in range(5)]
    res = run(ref, recs, long_read=long_read)
    assert res.status == 0
    kept = long_read == _abi.PG_NOT_LONG_READ or (ins_run, del_run) == (4, 3)
    mq1 = 61 if long_read == _abi.PG_NOT_LONG_READ else 9
    p, q = at(res, 50), at(res, 80)
    assert (p["ins"], int(res.ins_qual[49])) == ((5, 5 * mq1) if kept else (0, 0))
    assert (q["dels"], int(res.del_qual[79])) == ((5, 5 * mq1) if kept else (0, 0))


@pytest.mark.parametrize("stop,counted", [(81, True), (80, False)])
def test_H4_deletion_must_end_inside_the_region(stop, counted):
    """A deletion counts only when both its first and last loci are in the region
    (S/PileUpRegion.scala:166): loci 80-81 deleted by 5 reads (20M 2D 20M at 60;
    locus 79 differs from locus 81, so no left shift).  Region [41, 81] counts it at
    80; region [41, 80] does not, while the reads' trusted M bases still count."""
    ref = list(rand_ref(120, seed=22))
    while ref[78] == ref[80]:
        ref[78] = "ACGT"[("ACGT".index(ref[78]) + 1) % 4]
    ref = "".join(ref)
    recs = [read(60, [(20, "M"), (2, "D"), (20, "M")], ref[59:79] + ref[81:101]) for _ in range(5)]
    st = build_store(recs)
    res = oracle.process_region(st, _abi.default_params(), ref_from(ref), 0, 41, stop)
    assert res.status == 0
    assert at(res, 80, start=41)["dels"] == (5 if counted else 0)
    assert sum(at(res, 79, start=41)["count"]) == 5


@pytest.mark.parametrize("start,counted", [(41, True), (42, False)])
def test_H4_insertion_locus_checked_before_shift(start, counted):
    """An insertion counts when its pre-shift locus is in the region
    (S/PileUpRegion.scala:155): "G" inserted before locus 41 (20M 1I 20M at 21,
    locus 40 is not 'G', so it stays at 41) counts at 41 in a region starting at 41
    and nowhere in one starting at 42."""
    ref = list(rand_ref(120, seed=23))
    if ref[39] == "G":
        ref[39] = "T" if ref[38] != "T" and ref[40] != "T" else "A"
    ref = "".join(ref)
    assert ref[39] != "G"
    recs = [read(21, [(20, "M"), (1, "I"), (20, "M")], ref[20:40] + "G" + ref[40:60]) for _ in range(5)]
    st = build_store(recs)
    res = oracle.process_region(st, _abi.default_params(), ref_from(ref), 0, start, 100)
    assert res.status == 0
    assert int(res.insertions.sum()) == (5 if counted else 0)
    if counted:
        assert at(res, 41, start=start)["ins"] == 5


@pytest.mark.parametrize("start,ins_run,kept", [(1, 5, True), (31, 5, False), (31, 3, True)])
def test_long_read_deletion_run_is_read_at_the_region_index(start, ins_run, kept):
    """The long-read deletion test homoRun(index(dloc)) (S/PileUpRegion.scala:178)
    passes the region index dloc - start as a contig index.  Locus 80 deleted
    inside a T run of 3 (kept on its own); with the region starting at 31 the run
    measured is the one at contig index 49, locus 50: the C run of ins_run bases
    there (5 -> dropped, 3 -> kept)."""
    ref = _long_read_ref(ins_run, 3)
    recs = [read(60, [(20, "M"), (1, "D"), (20, "M")], ref[59:79] + ref[80:100]) for _ in range(5)]
    st = build_store(recs)
    res = oracle.process_region(st, _abi.default_params(long_read=_abi.PG_PACBIO), ref_from(ref), 0, start, 120)
    assert res.status == 0
    assert at(res, 80, start=start)["dels"] == (5 if kept else 0)


def test_H8_non_acgt_and_low_quality_bases():
    """PileUp.add (S/PileUp.scala:75-84) drops bases outside ACGT and bases below
    minQual, but PileUpRegion.add (S/PileUpRegion.scala:38-47) counts every valid
    trusted base in the region's baseCount first.  One 40M read at 101 (trusted
    loci 111..130) with N at 115, IUPAC R at 116, '=' at 117 and quality 5 at 118,
    minQual 10: those four loci stay empty; baseCount = 20."""
    ref = rand_ref(200, seed=31)
    seq = list(ref[100:140])
    seq[14], seq[15], seq[16] = "N", "R", "="
    qual = [30] * 40
    qual[17] = 5
    res = run(ref, [read(101, [(40, "M")], "".join(seq), qual=qual)], min_qual=10)
    assert res.status == 0 and res.stats.base_count == 20
    for locus in (115, 116, 117, 118):
        p = at(res, locus)
        assert p["count"] == [0, 0, 0, 0] and p["mq"] == 0 and p["q"] == 0
    b = "ACGT".index(ref[118])
    p = at(res, 119)
    assert p["count"][b] == 1 and p["qual_sum"][b] == 30 * 61 and p["mq"] == 61


def test_H8_indel_string_with_N_is_not_called():
    """hetIndelCall rejects a winning indel string that contains N
    (S/PileUp.scala:219): 8 of 10 reads insert "NA" before 51, which would be a
    homozygous insertion as "CA" is; the insertions still count."""
    ref, res = _ins_case(8, 2, ins="NA")
    p = at(res, 51)
    assert p["ins"] == 8
    assert not p["call"] & _abi.PG_CALL_INS and (p["call"] >> 9) & 7 == _abi.PG_CHANGE_NONE
    ref, res = _ins_case(8, 2, ins="CA")
    assert at(res, 51)["call"] & _abi.PG_CALL_INS


def _tile_reads(ref, snps=None, ins=None, dels=None, length=60, step=2):
    """Reads of `length` bases starting every `step` loci, carrying the sample's
    edits with matching CIGARs: snps {locus: base}, ins {locus: bases inserted
    before locus}, dels {first locus: last locus}.  Reads start on a plain
    reference base and end inside an M run, as an aligner would place them.
    Returns (records, sample sequence)."""
    snps, ins, dels = snps or {}, ins or {}, dels or {}
    sample, loc = [], 1
    while loc <= len(ref):
        if loc in ins:
            sample.append(ins[loc])
        if loc in dels:
            loc = dels[loc] + 1
            continue
        sample.append(snps.get(loc, ref[loc - 1]))
        loc += 1
    deleted = {x for a, b in dels.items() for x in range(a, b + 1)}
    recs = []
    for p in range(1, len(ref) + 1, step):
        if p in deleted or p in ins:
            continue
        cigar, seq, loc = [], "", p
        while len(seq) < length and loc <= len(ref):
            if loc > p and loc in ins:
                cigar.append((len(ins[loc]), "I"))
                seq += ins[loc]
                if len(seq) >= length:
                    break
            if loc > p and loc in dels:
                cigar.append((dels[loc] - loc + 1, "D"))
                loc = dels[loc] + 1
                continue
            if cigar and cigar[-1][1] == "M":
                cigar[-1] = (cigar[-1][0] + 1, "M")
            else:
                cigar.append((1, "M"))
            seq += snps.get(loc, ref[loc - 1])
            loc += 1
        if len(seq) != length or cigar[-1][1] != "M":
            continue
        recs.append(read(p, cigar, seq))
    return recs, "".join(sample)


def test_changes_offsets_across_region_chunks():
    """A 700-bp contig polished in two 350-bp regions (GenomeFile.contigRegions,
    S/GenomeFile.scala:67-74).  writeChanges (S/GenomeRegion.scala:645-657) adds
    the delta of the region's earlier fixes, and GenomeFile adds the length
    change of the contig's earlier regions as the offset (S/GenomeFile.scala:150-153):
      chr1:101 chr1_pilon:101-102 . CA           region 1, offset 0
      chr1:501-502 chr1_pilon:503 r501r502 .     region 2, offset +2, delta 0
      chr1:600 chr1_pilon:600 r600 s             offset +2, delta -2
    The FASTA joins the two fixed regions into the sample sequence."""
    ref = list(rand_ref(700, seed=12))
    if ref[99] == "A":   # locus 100 is not 'A': the insertion does not shift
        ref[99] = "T" if ref[98] != "T" and ref[100] != "T" else "G"
    while ref[499] == ref[501]:  # locus 500 differs from locus 502: the deletion does not shift
        ref[499] = "ACGT"[("ACGT".index(ref[499]) + 1) % 4]
    ref = "".join(ref)
    assert ref[99] != "A" and ref[98] != ref[99] != ref[100]
    snp = "ACGT"[("ACGT".index(ref[599]) + 2) % 4]
    recs, sample = _tile_reads(ref, snps={600: snp}, ins={101: "CA"}, dels={501: 502})
    st = build_store(recs)
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "o")
        assert oracle.polish(st, _abi.default_params(), ["chr1"], [ref_from(ref)], pre, chunk_size=350) == 0
        ch = open(pre + ".changes").read().splitlines()
        fa = "".join(open(pre + ".fasta").read().splitlines()[1:])
    assert ch == ["chr1:101 chr1_pilon:101-102 . CA", f"chr1:501-502 chr1_pilon:503 {ref[500:502]} .",
                  f"chr1:600 chr1_pilon:600 {ref[599]} {snp}"]
    assert fa == sample and len(fa) == 700


@pytest.mark.parametrize("long_read,start,zeroed", [(_abi.PG_NANOPORE, 1, 50), (_abi.PG_NANOPORE, 31, 80),
                                                    (_abi.PG_PACBIO, 1, None)])
def test_nanopore_motif_quality_zero(long_read, start, zeroed):
    """Nanopore reads add the base at the centre of a CC?GG motif with quality 0
    (S/PileUpRegion.scala:128-134, 189).  nanoporeExclude(index(locus)) reads the
    contig at the region index: with the motif centred on locus 50, a region
    starting at 1 zeroes locus 50, one starting at 31 zeroes locus 80 (index 49)
    and not 50.  PacBio reads keep their qualities.  Ten reads 40M at 31 and at
    61, quality 30, mapq 60: a zeroed locus has count 10, qualSum 0, mqSum 610."""
    ref = list(rand_ref(120, seed=41))
    ref[47:52] = "CCAGG"
    ref = "".join(ref)
    motif = lambda c: ref[c - 3] == "C" and ref[c - 2] == "C" and ref[c] == "G" and ref[c + 1] == "G"
    assert motif(50) and not motif(80) and not motif(20)
    recs = [read(31, [(40, "M")], ref[30:70]) for _ in range(10)]
    recs += [read(61, [(40, "M")], ref[60:100]) for _ in range(10)]
    res = run(ref, recs, start=start, long_read=long_read)
    assert res.status == 0
    for locus in (50, 80):
        p = at(res, locus, start=start)
        b = "ACGT".index(ref[locus - 1])
        assert p["count"][b] == 10 and p["mq"] == 610
        assert p["qual_sum"][b] == (0 if locus == zeroed else 10 * 30 * 61), locus


@pytest.mark.parametrize("snp_locus,fixed", [(61, False), (62, True), (40, True)])
def test_long_read_only_excludes_run_starts(snp_locus, fixed):
    """With long reads only, excludeMotifs (S/GenomeRegion.scala:416-439) marks
    the loci whose forward reference run (to the region's end) has 4 or more
    bases, and identifyAndFixIssues skips their changes (S/GenomeRegion.scala:326).
    In an A run at loci 60-64 that is 60 (run 5) and 61 (run 4), not 62 (run 3):
    a homozygous SNP at 61 is not fixed, one at 62 or outside the run is."""
    ref = list(rand_ref(120, seed=43))
    ref[58], ref[59:64], ref[64] = "C", "AAAAA", "G"
    ref = "".join(ref)
    snp = "T" if ref[snp_locus - 1] != "T" else "G"
    recs, sample = _tile_reads(ref, snps={snp_locus: snp}, length=40, step=1)
    st = build_store(recs)
    params = _abi.default_params(long_read=_abi.PG_PACBIO, long_read_only=1)
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "o")
        assert oracle.polish(st, params, ["chr1"], [ref_from(ref)], pre) == 0
        ch = open(pre + ".changes").read().splitlines()
        fa = "".join(open(pre + ".fasta").read().splitlines()[1:])
    if fixed:
        assert ch == [f"chr1:{snp_locus} chr1_pilon:{snp_locus} {ref[snp_locus - 1]} {snp}"] and fa == sample
    else:
        assert ch == [] and fa == ref


def test_placed_unmapped_read():
    """queryOverlapping returns an unmapped read placed inside the window, and
    htsjdk's getAlignmentEnd is 0 for it.  addRead (S/PileUpRegion.scala:102-220)
    piles nothing (no CIGAR) but counts the read, and physCovIncr(150, 0, ...) for
    an unpaired valid read (mapq 0 >= minMq 0) covers [min(150, 0), max) = [0, 150):
    the start lies before the region, so physCovStart += 1 and insertSizeStart +=
    150, and position 150 takes them back (S/PileUpRegion.scala:62-100).  So loci
    1-149 get physical coverage 1 and insert size 150, and addInsert counts an FR
    insert of 150 (S/BamFile.scala:137, 194-202)."""
    ref = rand_ref(300, seed=44)
    st = build_store([read(150, [], "ACGTACGTAC", mapq=0, flag=0x4)])
    assert st.aend[0] == 0
    res = oracle.process_region(st, _abi.default_params(), ref_from(ref), 0, 1, 300)
    assert res.status == 0
    assert res.stats.read_count == 1 and res.stats.base_count == 0
    assert res.stats.phys_cov_start == 1 and res.stats.insert_size_start == 150
    assert at(res, 1)["pc"] == 1 and at(res, 149)["pc"] == 1 and at(res, 150)["pc"] == 0
    assert at(res, 1)["isz"] == 150 and at(res, 150)["isz"] == 0
    assert (res.stats.fr_count, res.stats.fr_sum) == (1, 150) and res.stats.rf_count == 0
    assert int(res.count.sum()) == 0


@pytest.mark.parametrize("base,shifted", [("A", True), ("a", False)])
def test_soft_masked_reference_compares_raw(base, shifted):
    """Soft-masked (lowercase) reference bytes: the insertion left shift
    compares them raw with the read's bases (S/PileUpRegion.scala:156), so
    "CA" inserted before 51 shifts to 50 after an 'A' at 50 but not after an 'a';
    reference bases elsewhere are upper-cased (refBase, S/GenomeRegion.scala:783-787),
    and the polished FASTA keeps the file's case where nothing is fixed."""
    ref = list(rand_ref(100, seed=3))
    ref[48] = "G" if ref[47] != "G" else "T"   # locus 49 stops a shift past 50
    ref[49] = base
    ref = "".join(ref)
    seqref = ref.upper()
    recs = [read(31, [(20, "M"), (2, "I"), (20, "M")], seqref[30:50] + "CA" + seqref[50:70]) for _ in range(8)]
    recs += [read(31, [(40, "M")], seqref[30:70]) for _ in range(2)]
    res = run(ref, recs)
    assert res.status == 0
    at_locus = 50 if shifted else 51
    assert at(res, at_locus)["ins"] == 8 and at(res, 101 - at_locus)["ins"] == 0
    if not shifted:
        low = ref.lower()
        st = build_store(recs)
        with tempfile.TemporaryDirectory() as d:
            pre = os.path.join(d, "o")
            assert oracle.polish(st, _abi.default_params(), ["chr1"], [ref_from(low)], pre) == 0
            fa = "".join(open(pre + ".fasta").read().splitlines()[1:])
        assert fa == low[:50] + "CA" + low[50:]  # the homozygous insertion is fixed; the rest keeps its case
