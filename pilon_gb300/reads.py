"""Packed structure-of-arrays read store.

The fields are the htsjdk SAMRecord getters that Pilon's hot path reads
(S/PileUpRegion.scala:103-115, S/BamFile.scala:101-105 and 137,
S/Assembler.scala:56-64), laid out as the pg_reads struct of the C ABI.
"""
from dataclasses import dataclass, field
import numpy as np

from . import _abi

NIB = "=ACMGRSVTWYHKDBN"
NIB_OF = {c: i for i, c in enumerate(NIB)}
BASE_NIB = np.array([1, 2, 4, 8], dtype=np.uint8)  # A C G T as BAM 4-bit codes

CIGAR_OPS = "MIDNSHP=X"
OP_M, OP_I, OP_D, OP_N, OP_S, OP_H, OP_P, OP_EQ, OP_X = range(9)


@dataclass
class ReadStore:
    pos: np.ndarray            # int32, 1-based alignment start
    aend: np.ndarray           # int32, alignment end
    flag: np.ndarray           # uint16
    mapq: np.ndarray           # uint8
    tlen: np.ndarray           # int32
    ref_id: np.ndarray         # int32
    mate_ref_id: np.ndarray    # int32
    cigar_off: np.ndarray      # int64
    n_cigar: np.ndarray        # uint16
    cigar: np.ndarray          # uint32
    seq_off: np.ndarray        # int64
    l_seq: np.ndarray          # int32
    seq: np.ndarray            # uint8, 4-bit codes, two per byte
    qual_off: np.ndarray       # int64
    qual: np.ndarray           # uint8
    # getReadName as an id (mates share one); optional, host side only: the
    # stray-mate recruitment of local reassembly pairs reads by name
    name_id: np.ndarray = None  # int64
    _keep: list = field(default_factory=list, repr=False)

    @property
    def n_reads(self):
        return int(self.pos.shape[0])

    def aligned_bases(self):
        """M/=/X bases per read (the unit of the throughput metric)."""
        ops = self.cigar & 15
        lens = (self.cigar >> 4).astype(np.int64)
        m = np.where((ops == OP_M) | (ops == OP_EQ) | (ops == OP_X), lens, 0)
        csum = np.concatenate([[0], np.cumsum(m)])
        return csum[self.cigar_off + self.n_cigar] - csum[self.cigar_off]

    def nbytes(self):
        return sum(getattr(self, f).nbytes for f in FIELDS)

    def to_abi(self):
        """pg_reads struct with host pointers into this store's arrays."""
        arrs = {}
        for f in FIELDS:
            a = np.ascontiguousarray(getattr(self, f), dtype=DTYPES[f])
            arrs[f] = a
        self._keep = list(arrs.values())
        r = _abi.pg_reads()
        r.n_reads = self.n_reads
        for f in FIELDS:
            setattr(r, f, arrs[f].ctypes.data if arrs[f].size else 0)
        r.n_cigar_words = int(arrs["cigar"].size)  # the packed upload checks the lengths against these
        r.seq_bytes = int(arrs["seq"].size)
        r.qual_bytes = int(arrs["qual"].size)
        return r

    # ---- per-read accessors (test helpers) ----
    def read_bases(self, i):
        n = int(self.l_seq[i])
        o = int(self.seq_off[i])
        b = self.seq[o:o + (n + 1) // 2]
        nib = np.empty(2 * b.size, dtype=np.uint8)
        nib[0::2] = b >> 4
        nib[1::2] = b & 15
        return "".join(NIB[x] for x in nib[:n])

    def read_cigar(self, i):
        o = int(self.cigar_off[i])
        return [(int(w >> 4), CIGAR_OPS[int(w & 15)]) for w in self.cigar[o:o + int(self.n_cigar[i])]]

    def cigar_string(self, i):
        return "".join(f"{n}{op}" for n, op in self.read_cigar(i)) or "*"

    def subset(self, idx):
        """A new store holding reads `idx` (in that order)."""
        idx = np.asarray(idx, dtype=np.int64)
        nc = self.n_cigar[idx].astype(np.int64)
        co = np.concatenate([[0], np.cumsum(nc)])[:-1]
        cig = np.concatenate([self.cigar[self.cigar_off[i]:self.cigar_off[i] + nc[k]]
                              for k, i in enumerate(idx)]) if idx.size else np.zeros(0, np.uint32)
        sb = ((self.l_seq[idx].astype(np.int64) + 1) // 2)
        so = np.concatenate([[0], np.cumsum(sb)])[:-1]
        seq = np.concatenate([self.seq[self.seq_off[i]:self.seq_off[i] + sb[k]]
                              for k, i in enumerate(idx)]) if idx.size else np.zeros(0, np.uint8)
        qb = self.l_seq[idx].astype(np.int64)
        qo = np.concatenate([[0], np.cumsum(qb)])[:-1]
        qual = np.concatenate([self.qual[self.qual_off[i]:self.qual_off[i] + qb[k]]
                               for k, i in enumerate(idx)]) if idx.size else np.zeros(0, np.uint8)
        return ReadStore(self.pos[idx].copy(), self.aend[idx].copy(), self.flag[idx].copy(),
                         self.mapq[idx].copy(), self.tlen[idx].copy(), self.ref_id[idx].copy(),
                         self.mate_ref_id[idx].copy(), co.astype(np.int64), nc.astype(np.uint16),
                         cig.astype(np.uint32), so.astype(np.int64), self.l_seq[idx].copy(),
                         seq.astype(np.uint8), qo.astype(np.int64), qual.astype(np.uint8),
                         None if self.name_id is None else self.name_id[idx].copy())


FIELDS = ["pos", "aend", "flag", "mapq", "tlen", "ref_id", "mate_ref_id", "cigar_off", "n_cigar",
          "cigar", "seq_off", "l_seq", "seq", "qual_off", "qual"]
DTYPES = {"pos": np.int32, "aend": np.int32, "flag": np.uint16, "mapq": np.uint8, "tlen": np.int32,
          "ref_id": np.int32, "mate_ref_id": np.int32, "cigar_off": np.int64, "n_cigar": np.uint16,
          "cigar": np.uint32, "seq_off": np.int64, "l_seq": np.int32, "seq": np.uint8,
          "qual_off": np.int64, "qual": np.uint8}


def encode_seq(s):
    """String of read bases -> packed 4-bit bytes (BAM layout)."""
    nib = np.array([NIB_OF[c] for c in s], dtype=np.uint8)
    if nib.size % 2:
        nib = np.concatenate([nib, [0]]).astype(np.uint8)
    return ((nib[0::2] << 4) | nib[1::2]).astype(np.uint8)


def cigar_words(ops):
    """[(len, 'M'), ...] -> uint32 BAM CIGAR words."""
    return np.array([(n << 4) | CIGAR_OPS.index(op) for n, op in ops], dtype=np.uint32)


def build_store(records):
    """ReadStore from a list of dicts (pos, cigar [(n,op)], seq str, qual list|None,
    flag, mapq, tlen, ref_id, mate_ref_id).  Used for hand-made test cases."""
    n = len(records)
    cig, seqb, qualb = [], [], []
    co, so, qo = [], [], []
    c = s = q = 0
    aend = []
    for r in records:
        w = cigar_words(r["cigar"])
        co.append(c); c += w.size; cig.append(w)
        sb = encode_seq(r["seq"])
        so.append(s); s += sb.size; seqb.append(sb)
        L = len(r["seq"])
        qa = np.full(L, 0xFF, np.uint8) if r.get("qual") is None else np.array(r["qual"], np.uint8)
        qo.append(q); q += L; qualb.append(qa)
        rl = sum(k for k, op in r["cigar"] if op in "MDN=X")
        # htsjdk getAlignmentEnd: 0 for an unmapped read, else start + reference
        # length - 1 (start - 1 when no operator consumes the reference)
        aend.append(0 if r.get("flag", 0) & 0x4 else r["pos"] + rl - 1)
    cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)
    return ReadStore(
        pos=np.array([r["pos"] for r in records], np.int32),
        aend=np.array(aend, np.int32),
        flag=np.array([r.get("flag", 0) for r in records], np.uint16),
        mapq=np.array([r.get("mapq", 60) for r in records], np.uint8),
        tlen=np.array([r.get("tlen", 0) for r in records], np.int32),
        ref_id=np.array([r.get("ref_id", 0) for r in records], np.int32),
        mate_ref_id=np.array([r.get("mate_ref_id", r.get("ref_id", 0)) for r in records], np.int32),
        cigar_off=np.array(co, np.int64), n_cigar=np.array([len(r["cigar"]) for r in records], np.uint16),
        cigar=cat(cig, np.uint32), seq_off=np.array(so, np.int64),
        l_seq=np.array([len(r["seq"]) for r in records], np.int32), seq=cat(seqb, np.uint8),
        qual_off=np.array(qo, np.int64), qual=cat(qualb, np.uint8),
        name_id=(np.array([r["name"] for r in records], np.int64) if records and "name" in records[0] else None))


def concat_stores(stores):
    """Concatenate read stores (offsets rebased)."""
    cig_base = np.cumsum([0] + [s.cigar.size for s in stores])[:-1]
    seq_base = np.cumsum([0] + [s.seq.size for s in stores])[:-1]
    qual_base = np.cumsum([0] + [s.qual.size for s in stores])[:-1]
    cat = np.concatenate
    names = None
    if all(s.name_id is not None for s in stores):
        # read names stay distinct across the stores (as the names of one BAM)
        base = np.cumsum([0] + [int(s.name_id.max()) + 1 if s.n_reads else 0 for s in stores])[:-1]
        names = cat([s.name_id + b for s, b in zip(stores, base)]).astype(np.int64)
    return ReadStore(
        cat([s.pos for s in stores]), cat([s.aend for s in stores]), cat([s.flag for s in stores]),
        cat([s.mapq for s in stores]), cat([s.tlen for s in stores]), cat([s.ref_id for s in stores]),
        cat([s.mate_ref_id for s in stores]),
        cat([s.cigar_off + b for s, b in zip(stores, cig_base)]), cat([s.n_cigar for s in stores]),
        cat([s.cigar for s in stores]),
        cat([s.seq_off + b for s, b in zip(stores, seq_base)]), cat([s.l_seq for s in stores]),
        cat([s.seq for s in stores]),
        cat([s.qual_off + b for s, b in zip(stores, qual_base)]), cat([s.qual for s in stores]), names)


def merge_sorted(stores):
    """One coordinate-sorted store from several (the BAMs of one type that
    Pilon reads one after another into the same pileups, S/GenomeRegion.scala:
    287-300): reads ordered by reference, the unplaced reads (reference -1)
    last, then by position, ties kept in input order.  Within one BAM type the
    pileups, calls and region statistics do not depend on the order reads are
    added, so the merged store gives the same results; the insert-size
    statistics come out summed over the BAMs instead of per BAM."""
    cat = concat_stores(stores)
    rid = cat.ref_id.astype(np.int64)
    key_ref = np.where(rid < 0, np.int64(1) << 40, rid)
    order = np.lexsort((np.arange(cat.n_reads), cat.pos.astype(np.int64), key_ref))
    return cat.subset(order)
