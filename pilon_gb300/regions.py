"""Region partitioning and the read range fed to each region.

contig_regions restates GenomeFile.contigRegions (S/GenomeFile.scala:67-74);
read ranges reproduce the window of BamFile.process
(S/BamFile.scala:117-119): every read overlapping
[max(start-10000, 0), min(stop+10000, len)] is fed to the region.
"""
import numpy as np

SLOP = 10000


def contig_regions(contig_len, chunk_size=10_000_000):
    """[(start, stop)] 1-based closed chunks of one contig."""
    n_chunks = (contig_len + chunk_size - 1) // chunk_size
    cs = (contig_len + n_chunks - 1) // n_chunks
    return [(b, min(contig_len, b + cs - 1)) for b in range(1, contig_len + 1, cs)]


def parse_targets(target_string, names, lens):
    """--targets (S/GenomeFile.scala:239-249): a file whose lines are target
    strings, or else the argument itself as one.  As in the reference, any error
    while reading or parsing the file (a missing file, a bad or blank line) makes
    it fall back to parsing the argument as a target string."""
    try:
        with open(target_string) as f:
            lines = f.read().splitlines()
        out = [t for line in lines for t in parse_target_string(line, names, lens)]
    except Exception:
        out = []
    return out or parse_target_string(target_string, names, lens)


def parse_target_string(target_string, names, lens):
    """"name:start-stop,..." or whole contigs (S/GenomeFile.scala:215-236)."""
    import re
    out = []
    for t in target_string.split(","):
        m = re.match(r"^\s*(.+):([0-9]+)-([0-9]+)\s*$", t)
        if m:
            name, s, e = m.group(1), int(m.group(2)), int(m.group(3))
        else:
            name = t
            s, e = 1, int(lens[names.index(t)])
        ci = names.index(name)
        if e > lens[ci]:
            raise ValueError("GenomeRegion stop point must be within contig")
        out.append((ci, s, e))
    return out


class ReadIndex:
    """Locates the reads of each contig in a (ref_id, pos)-sorted store."""

    def __init__(self, reads, n_contigs):
        self.reads = reads
        rid = reads.ref_id
        # A coordinate-sorted BAM ends with its unplaced reads (reference -1),
        # which no region query returns; the placed reads before them are
        # sorted by reference.
        # one past the last placed read (found from the end, without listing every placed read)
        tail_placed = rid[::-1] >= 0
        m = rid.size - int(np.argmax(tail_placed)) if rid.size and bool(tail_placed.any()) else 0
        head = rid[:m]
        if m and (int(head.min()) < 0 or bool(np.any(head[1:] < head[:-1]))):
            raise ValueError("reads are not coordinate-sorted: unplaced reads (reference -1) must come last")
        # search keys in the arrays' own types: an int64 key would widen the whole array per search
        ids = np.arange(n_contigs, dtype=head.dtype)
        self.contig_lo = np.searchsorted(head, ids, side="left")
        self.contig_hi = np.searchsorted(head, ids, side="right")
        self.max_span = int((reads.aend[:m] - reads.pos[:m]).max()) + 1 if m else 0

    def range_for(self, contig, start, stop, contig_len, slop=SLOP):
        lo, hi = int(self.contig_lo[contig]), int(self.contig_hi[contig])
        qs = max(start - slop, 0)
        qe = min(stop + slop, contig_len)
        pos = self.reads.pos[lo:hi]
        key = pos.dtype.type
        a = lo + int(np.searchsorted(pos, key(max(qs - self.max_span, np.iinfo(pos.dtype).min)), side="left"))
        b = lo + int(np.searchsorted(pos, key(min(qe, np.iinfo(pos.dtype).max)), side="right"))
        return a, b


def plan_regions(reads, contig_lens, chunk_size=10_000_000, targets=None, order=None):
    """[(contig, start, stop, read_begin, read_end)] in processing order: the
    targets, or the chunks of every contig in `order` (contig indices; all of
    them in index order by default)."""
    idx = ReadIndex(reads, len(contig_lens))
    regs = []
    if targets is not None:
        for ci, s, e in targets:
            a, b = idx.range_for(ci, s, e, contig_lens[ci])
            regs.append((ci, s, e, a, b))
        return regs
    for ci in (range(len(contig_lens)) if order is None else order):
        ln = contig_lens[ci]
        for s, e in contig_regions(int(ln), chunk_size):
            a, b = idx.range_for(ci, s, e, int(ln))
            regs.append((ci, s, e, a, b))
    return regs
