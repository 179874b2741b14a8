"""Local reassembly for the fix types gaps and local: the host side that
Pilon's GenomeRegion.identifyAndFixIssues runs around GapFiller
(S/GenomeRegion.scala:382-410).

  BamFile.scan                 whole-store insert statistics and stray mates (numpy)
  GapFiller.recruitReads       reads overlapping a break's flanks plus their stray mates (numpy)
  Assembler.addReads/build     pg_kmer_tally_reads, every window of every region in one device call
  graph walk, GapFiller        pg_reassemble (C++, host threads)

The read store must be coordinate-sorted, with read names given as ids in
`reads.name_id` (mates share one) for the stray mates; without them the
recruitment is that of --nostrays.
"""
import numpy as np

from . import _abi
from .engine import scan_reads

MAX_INSERT_DEFAULT = {_abi.PG_BAM_FRAGS: 500, _abi.PG_BAM_JUMPS: 10000, _abi.PG_BAM_UNPAIRED: 10000,
                      _abi.PG_BAM_BAM: 10000}  # BamFile.maxInsertSizes (S/BamFile.scala:29)


def validate(flag, params):
    """BamFile.validateRead (S/BamFile.scala:101-105) over a flag array."""
    ok = (flag & 0x100) == 0
    if not params.nonpf:
        ok &= (flag & 0x200) == 0
    if not params.duplicates:
        ok &= (flag & 0x400) == 0
    return ok


def _wrap32(x):
    return ((x + (1 << 31)) % (1 << 32)) - (1 << 31)


class InsertStats:
    """BamFile.InsertSizeStats (S/BamFile.scala:156-186)."""

    def __init__(self, count=0, total=0, sumsq=0):
        self.count, self.sum, self.sumsq = int(count), int(total), int(sumsq)

    def add(self, count, total, sumsq):
        self.count += int(count)
        self.sum += int(total)
        self.sumsq += int(sumsq)

    def mean(self):
        return self.sum / self.count if self.count > 0 else 0.0

    def sigma(self):
        if self.sum > 0:
            m = self.mean()
            return abs(self.sumsq / self.count - m * m) ** 0.5
        return 0.0

    def max_insert_size(self):
        return _java_l2i(_java_round(self.mean() + 3.0 * self.sigma())) if self.count > 1000 else 0


def _java_round(x):
    """java.lang.Math.round(double): floor(x + 0.5), NaN -> 0, saturating."""
    import math
    if x != x:
        return 0
    r = math.floor(x + 0.5)
    return max(min(r, (1 << 63) - 1), -(1 << 63))


def _java_l2i(x):
    return _wrap32(int(x))


def _pct(n, d):  # Utils.pct on Longs (S/Utils.scala:23-25)
    return (100 * n + d // 2) // d if d > 0 else 0


class BamState:
    """One BAM's state that local reassembly reads: the insert statistics of
    BamFile.scan plus those of every region processed so far, and the
    strayMateMap (S/BamFile.scala:156-337)."""

    def __init__(self, reads, params, n_contigs, strays=True):
        self.reads, self.params = reads, params
        self.bam_type = int(params.bam_type)
        self.huge = 5 * MAX_INSERT_DEFAULT[self.bam_type]
        self.fr, self.rf, self.un = InsertStats(), InsertStats(), InsertStats()
        self.strays = bool(strays) and reads.name_id is not None
        flag = reads.flag  # uint16: the bit tests need no wider copy
        self.valid = validate(flag, params)
        unmapped = (flag & 0x4) != 0
        # the insert statistics (proper pairs by inferred insert size, unpaired reads by length) and
        # the stray-mate candidates (paired, not proper, mate mapped, on a reference of interest) of
        # BamFile.scan: one pass on host threads (pg_scan_reads)
        stats, first, second = scan_reads(reads, params, n_contigs, self.huge, strays=self.strays)
        self.fr.add(*stats[0:3])
        self.rf.add(*stats[3:6])
        self.un.add(*stats[6:9])
        self._stray = [(np.zeros(0, np.int64), np.zeros(0, np.int64))] * 2
        if self.strays:
            self._stray = [self._name_map(first), self._name_map(second)]
        # each contig's reads and the longest alignment span among them
        self.n_contigs = n_contigs
        rid = reads.ref_id
        unplaced = np.nonzero(rid < 0)[0]  # the unplaced reads close a coordinate-sorted store
        placed = rid[:int(unplaced[0])] if unplaced.size else rid
        ids = np.arange(n_contigs, dtype=placed.dtype)  # keys of the ids' own type: no widened copy
        self.cb = np.searchsorted(placed, ids, side="left").astype(np.int64)
        self.ce = np.searchsorted(placed, ids, side="right").astype(np.int64)
        self.pos = reads.pos.astype(np.int64)  # searched with int64 bounds without a cast per search
        self.end = np.where(unmapped, reads.pos, reads.aend).astype(np.int64)
        span = self.end - self.pos + 1
        self.span = np.array([int(span[a:b].max()) if b > a else 1 for a, b in zip(self.cb, self.ce)], np.int64)

    def _name_map(self, idx):
        """HashMap name -> read of MateMap.addRead, the last read of a name
        winning: (sorted names, reads)."""
        names = self.reads.name_id[idx]
        order = np.lexsort((idx, names))
        names, idx = names[order], idx[order]
        last = np.ones(names.size, bool)
        last[:-1] = names[1:] != names[:-1]
        return names[last], idx[last]

    def add_region(self, st):
        """The insert sizes BamFile.process adds for one region (pg_region_stats)."""
        self.fr.add(st.fr_count, st.fr_sum, st.fr_sumsq)
        self.rf.add(st.rf_count, st.rf_sum, st.rf_sumsq)

    def pct_fr(self):
        return _pct(self.fr.count, self.fr.count + self.rf.count + self.un.count)

    def insert_size_mean(self):  # S/BamFile.scala:208-210
        return self.fr.mean() if self.pct_fr() >= 50 else self.rf.mean()

    def max_insert_size(self):  # S/BamFile.scala:216-220
        m = max(self.fr.max_insert_size(), self.rf.max_insert_size(), self.un.max_insert_size())
        return m if m > 0 else MAX_INSERT_DEFAULT[self.bam_type]

    def break_radius(self, K):  # GapFiller.breakRadius (S/GapFiller.scala:357-362)
        mean = _java_l2i(_java_round(self.insert_size_mean())) if self.bam_type == _abi.PG_BAM_FRAGS else 0
        return max(3 * K, mean)

    def reads_in_region(self, contig, s, e):
        """BamFile.readsInRegion (S/BamFile.scala:339-344): htsjdk's
        queryOverlapping, the alignment [start, end] (end = start for an
        unmapped read) meeting [s, e], then validateRead."""
        a, b = int(self.cb[contig]), int(self.ce[contig])
        pos = self.pos
        lo = a + int(np.searchsorted(pos[a:b], np.int64(s - int(self.span[contig])), side="left"))
        hi = a + int(np.searchsorted(pos[a:b], np.int64(e), side="right"))
        idx = np.arange(lo, hi, dtype=np.int64)
        keep = (pos[lo:hi] <= e) & (self.end[lo:hi] >= s) & self.valid[lo:hi]
        return idx[keep]

    def recruit(self, contig, s, e):
        """GapFiller.recruitReads (S/GapFiller.scala:364-402) for this BAM:
        recruitFlankReads (S/BamFile.scala:346-364), with the stray mates of
        MateMap.findStrays (:244-257) after the flank reads."""
        if self.bam_type == _abi.PG_BAM_UNPAIRED and self.params.long_read:
            return np.zeros(0, np.int64)  # recruitUnpaired skips long reads
        if self.bam_type == _abi.PG_BAM_BAM:
            raise ValueError("local reassembly takes a BAM of type frags, jumps or unpaired")
        flank = self.max_insert_size()
        fs, fe = max(s - flank, 1), e + flank  # flankRegion (S/BamFile.scala:359-364)
        reads = self.reads_in_region(contig, fs, fe)
        if self.bam_type == _abi.PG_BAM_JUMPS:
            return self._bad_mates(reads, s, e, fs, fe)
        if not self.strays or self.bam_type == _abi.PG_BAM_UNPAIRED:
            return reads
        extra = self._find_strays(reads)
        return np.concatenate([reads, extra]) if extra.size else reads

    def _mate_map(self, reads):
        """MateMap.addRead (S/BamFile.scala:234-238): name -> read for the first
        and the other reads of pairs, the last read of a name winning; as
        (sorted names, reads) twice."""
        first = (self.reads.flag[reads] & 0x40) != 0
        return self._name_map(reads[first]), self._name_map(reads[~first])

    def _find_strays(self, reads):
        """MateMap(reads).findStrays (S/BamFile.scala:244-257): the strays' mates
        of the names that have one end among the reads (in HashMap order in the
        reference; sorted here, which the tally does not see)."""
        (m1, _), (m2, _) = self._mate_map(reads)
        found = []
        # a first-of-pair read's mate is looked up among the second-of-pair strays, and back
        for mine, other, table in ((m1, m2, self._stray[1]), (m2, m1, self._stray[0])):
            alone = np.setdiff1d(mine, other, assume_unique=True)
            tn, ti = table
            if alone.size and tn.size:
                k = np.minimum(np.searchsorted(tn, alone), tn.size - 1)
                found.append(ti[k[tn[k] == alone]])
        return np.sort(np.concatenate(found)) if found else np.zeros(0, np.int64)

    def _bad_mates(self, reads, s, e, fs, fe):
        """BamFile.recruitBadMates (S/BamFile.scala:366-403) for a jumps BAM: of
        each pair with both ends in the MateMap (with the strays' mates added),
        the mate of an end that is mapped, not in a proper pair, oriented
        towards the region's midpoint (when the BAM is almost all FR or RF)
        and inside the flanks."""
        r = self.reads
        if r.name_id is None:
            return np.zeros(0, np.int64)  # without names no pair is known
        if self.strays:
            reads = np.concatenate([reads, self._find_strays(reads)])  # MateMap.addStrays
        (n1, i1), (n2, i2) = self._mate_map(reads)
        both, k1, k2 = np.intersect1d(n1, n2, assume_unique=True, return_indices=True)
        a = np.concatenate([i1[k1], i2[k2]])  # pairs(): (read1, read2) and (read2, read1)
        b = np.concatenate([i2[k2], i1[k1]])
        fl = r.flag[a].astype(np.int64)
        rc = (fl & 0x10) != 0
        st, en = r.pos[a].astype(np.int64), r.aend[a].astype(np.int64)
        mid = (s + e) // 2
        fr = ((st < mid) & ~rc) | ((en > mid) & rc)
        pct = self.pct_fr()
        good = fr if pct > 90 else (~fr if pct < 10 else np.ones(a.size, bool))  # minOrientationPct 10
        keep = ((fl & 0x6) == 0) & good & (((st >= fs) & (st <= fe)) | ((en >= fs) & (en <= fe)))
        return np.sort(b[keep])


def gaps(ref, start, stop):
    """GenomeRegion.gaps (S/GenomeRegion.scala:700): runs of N in the
    reference (summaryRegions, slop 100, away from the region's ends), at
    least 10 bases long."""
    b = np.frombuffer(bytes(ref[start - 1:stop]).upper(), np.uint8) == ord("N")
    return [g for g in summary_regions(b, start, stop, 100) if g[1] + 1 - g[0] >= 10]


def summary_regions(test, start, stop, slop):
    """GenomeRegion.summaryRegions (S/GenomeRegion.scala:743-763) of a boolean
    array over the region."""
    idx = np.nonzero(test)[0]
    out = []
    if idx.size:
        # a run ends when a false position lies more than slop past its last
        # true one: the next true position is more than slop + 1 further on
        cut = np.nonzero(np.diff(idx) > slop + 1)[0]
        firsts = np.concatenate([[idx[0]], idx[cut + 1]])
        lasts = np.concatenate([idx[cut], [idx[-1]]])
        out = [(start + int(f), start + int(l)) for f, l in zip(firsts, lasts)]
    return [r for r in out if not (r[0] - start < 100 or stop - r[1] < 100)]
