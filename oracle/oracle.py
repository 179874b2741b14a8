"""ctypes wrapper of the CPU oracle (oracle/pilon_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, never by the pilon_gb300 product path.
Parity is unpinned by reference tests (the reference ships none); the oracle
is pinned by the hand-derived known-answer cases under tests/golden/.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from pilon_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or (os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "pilon_oracle.cpp"))):
            build()
        L = C.CDLL(LIB)
        L.or_process_region.restype = C.c_int
        L.or_process_region.argtypes = [C.POINTER(_abi.pg_reads), C.POINTER(_abi.pg_params), C.c_void_p, C.c_int64,
                                        C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.c_int64,
                                        C.POINTER(_abi.pg_region_out), C.POINTER(_abi.pg_region_stats)]
        L.or_contig_regions.restype = C.c_int32
        L.or_contig_regions.argtypes = [C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]
        L.or_polish.restype = C.c_int
        L.or_polish.argtypes = [C.POINTER(_abi.pg_reads), C.POINTER(_abi.pg_params), C.c_int32, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                C.c_int32, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                C.c_char_p, C.c_char_p]
        L.or_polish_fix.restype = C.c_int
        L.or_polish_fix.argtypes = L.or_polish.argtypes + [C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                                           C.c_void_p, C.c_int32, C.c_int32, C.c_int32]
        L.or_region_breaks.restype = C.c_int32
        L.or_region_breaks.argtypes = [C.POINTER(_abi.pg_reads), C.POINTER(_abi.pg_params), C.c_void_p, C.c_int64,
                                       C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.c_int64, C.c_void_p, C.c_int32]
        L.or_kmer_tally.restype = C.c_int64
        L.or_kmer_tally.argtypes = [C.POINTER(_abi.pg_reads), C.POINTER(_abi.pg_params), C.c_void_p, C.c_int32,
                                    C.c_int32, C.c_int32, C.c_void_p, C.c_int64]
        L.or_kmer_tally_wide.restype = C.c_int64
        L.or_kmer_tally_wide.argtypes = L.or_kmer_tally.argtypes
        L.or_target.restype = C.c_int
        L.or_target.argtypes = [C.POINTER(_abi.pg_reads), C.POINTER(_abi.pg_params), C.c_char_p, C.c_void_p,
                                C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.c_int64, C.c_int32,
                                C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_char_p, C.c_char_p, C.c_char_p]
        L.or_java_format2.restype = C.c_int
        L.or_java_format2.argtypes = [C.c_double, C.c_char_p, C.c_int]
        _lib = L
    return _lib


class RegionResult:
    """Arrays of one region, in the layout of pg_region_out."""
    FIELDS32 = ["mq_sum", "q_sum", "phys_cov", "insert_size", "bad_pair", "deletions", "del_qual",
                "insertions", "ins_qual", "clips", "indel_len", "ins_str"]

    def __init__(self, size, ins_cap=1 << 20):
        self.size = size
        self.count = np.zeros(4 * size, np.int32)
        self.qual_sum = np.zeros(4 * size, np.int64)
        for f in self.FIELDS32:
            setattr(self, f, np.zeros(size, np.int32))
        self.call = np.zeros(size, np.uint32)
        self.score = np.zeros(size, np.int64)
        self.ins_chars = np.zeros(ins_cap, np.uint8)
        self.stats = _abi.pg_region_stats()

    def out_struct(self):
        o = _abi.pg_region_out()
        o.count = self.count.ctypes.data
        o.qual_sum = self.qual_sum.ctypes.data
        for f in self.FIELDS32:
            setattr(o, f, getattr(self, f).ctypes.data)
        o.call = self.call.ctypes.data
        o.score = self.score.ctypes.data
        o.ins_chars = self.ins_chars.ctypes.data
        o.ins_chars_cap = self.ins_chars.size
        return o

    def insertion(self, i):
        off = int(self.ins_str[i])
        if off < 0:
            return ""
        return self.ins_chars[off:off + int(self.indel_len[i])].tobytes().decode()


def process_region(reads, params, contig, contig_id, start, stop, read_begin=0, read_end=None):
    """BamFile.process + GenomeRegion.postProcess for one region on the CPU."""
    L = lib()
    read_end = reads.n_reads if read_end is None else read_end
    contig = np.ascontiguousarray(contig, np.uint8)
    res = RegionResult(stop + 1 - start)
    ab = reads.to_abi()
    o = res.out_struct()
    rc = L.or_process_region(C.byref(ab), C.byref(params), contig.ctypes.data, contig.size, contig_id, start,
                             stop, read_begin, read_end, C.byref(o), C.byref(res.stats))
    res.status = rc
    return res


def contig_regions(contig_len, chunk_size=10_000_000):
    L = lib()
    cap = 4096
    s = np.zeros(cap, np.int32)
    e = np.zeros(cap, np.int32)
    n = L.or_contig_regions(contig_len, chunk_size, s.ctypes.data, e.ctypes.data, cap)
    return list(zip(s[:n].tolist(), e[:n].tolist()))


def polish(reads, params, names, contigs, out_prefix, chunk_size=10_000_000, fix_snps=True, fix_indels=True,
           iupac=False, diploid=False, vcf_qe=False, vcf_date="20260101", vcf_source="Pilon version [COMMIT] [DATE]",
           vcf_args="", vcf_ref="file:/genome.fasta", fix_gaps=False, fix_local=False, K=47, strays=True,
           stats=None, fix_breaks=False, vcf=True, gap_margin=100000, min_gap=10):
    """GenomeFile.processRegions with --fix snps,indels[,gaps,local] --vcf
    --changes; writes out_prefix.fasta / .vcf / .changes.  With gaps or local,
    K is --K and the stray mates come from reads.name_id (strays=False is
    --nostrays), fix_breaks is the experimental "breaks" fix, gap_margin and
    min_gap are --gapmargin and --mingap; stats (a dict)
    receives 'tied_sets'; vcf=False writes no VCF."""
    L = lib()
    n = len(contigs)
    arrs = [np.ascontiguousarray(c, np.uint8) for c in contigs]
    lens = np.array([a.size for a in arrs], np.int64)
    ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in arrs])
    nm = [s.encode() for s in names]
    nptrs = (C.c_char_p * n)(*nm)
    ab = reads.to_abi()
    args = (C.byref(ab), C.byref(params), n, C.cast(nptrs, C.c_void_p), lens.ctypes.data,
            C.cast(ptrs, C.c_void_p), chunk_size, int(fix_snps), int(fix_indels), int(iupac), int(diploid),
            int(vcf_qe), (out_prefix + ".fasta").encode(), (out_prefix + ".vcf").encode() if vcf else None,
            (out_prefix + ".changes").encode(), vcf_date.encode(), vcf_source.encode(), vcf_args.encode(),
            vcf_ref.encode())
    if not (fix_gaps or fix_local):
        return L.or_polish(*args)
    names_arr = None
    if strays and reads.name_id is not None:
        names_arr = np.ascontiguousarray(reads.name_id, np.int64)
    tied = C.c_int64(0)
    rc = L.or_polish_fix(*args, int(fix_gaps), int(fix_local), int(K),
                         names_arr.ctypes.data if names_arr is not None else None, C.byref(tied),
                         int(fix_breaks), int(gap_margin), int(min_gap))
    if stats is not None:
        stats["tied_sets"] = int(tied.value)
    return rc


def target(reads, params, name, contig, contig_id, start, stop, read_begin, read_end, fix_snps=True,
           fix_indels=True, iupac=False, diploid=False, vcf_qe=False):
    """`pilon --targets name:start-stop` on one region: returns (status, fixed
    bases, changes text, VCF records without header)."""
    import tempfile
    L = lib()
    contig = np.ascontiguousarray(contig, np.uint8)
    ab = reads.to_abi()
    with tempfile.TemporaryDirectory() as d:
        paths = [os.path.join(d, x) for x in ("bases", "changes", "vcf")]
        rc = L.or_target(C.byref(ab), C.byref(params), name.encode(), contig.ctypes.data, contig.size, contig_id,
                         start, stop, read_begin, read_end, int(fix_snps), int(fix_indels), int(iupac),
                         int(diploid), int(vcf_qe), *[x.encode() for x in paths])
        if rc:
            return rc, None, None, None
        return rc, open(paths[0], "rb").read(), open(paths[1]).read(), open(paths[2], "rb").read()


def region_breaks(reads, params, contig, contig_id, start, stop, read_begin=0, read_end=None):
    L = lib()
    read_end = reads.n_reads if read_end is None else read_end
    contig = np.ascontiguousarray(contig, np.uint8)
    cap = 1 << 16
    out = np.zeros(2 * cap, np.int32)
    ab = reads.to_abi()
    n = L.or_region_breaks(C.byref(ab), C.byref(params), contig.ctypes.data, contig.size, contig_id, start, stop,
                           read_begin, read_end, out.ctypes.data, cap)
    if n < 0:
        raise IndexError("reference would throw")
    return [(int(out[2 * k]), int(out[2 * k + 1])) for k in range(min(n, cap))]


def kmer_tally(reads, params, windows, K, min_depth=5):
    """Edges of Assembler.buildGraph per window (pg_kmer_edge records, 4-bit keys)."""
    L = lib()
    wins = (_abi.pg_window * max(1, len(windows)))(*[_abi.pg_window(a, b) for a, b in windows])
    ab = reads.to_abi()
    cap = 1
    while True:
        edges = np.zeros(cap, _abi.kmer_edge_dtype())
        n = L.or_kmer_tally(C.byref(ab), C.byref(params), C.cast(wins, C.c_void_p), len(windows), K, min_depth,
                            edges.ctypes.data, cap)
        if n <= cap:
            return edges[:n]
        cap = int(n)


def kmer_tally_wide(reads, params, windows, K, min_depth=5):
    """Edges of Assembler.buildGraph per window for any K <= 64
    (pg_kmer_edge_wide records, four words of 4-bit keys)."""
    L = lib()
    wins = (_abi.pg_window * max(1, len(windows)))(*[_abi.pg_window(a, b) for a, b in windows])
    ab = reads.to_abi()
    cap = 1
    while True:
        edges = np.zeros(cap, _abi.kmer_edge_wide_dtype())
        n = L.or_kmer_tally_wide(C.byref(ab), C.byref(params), C.cast(wins, C.c_void_p), len(windows), K, min_depth,
                                 edges.ctypes.data, cap)
        if n <= cap:
            return edges[:n]
        cap = int(n)


def java_format2(x):
    buf = C.create_string_buffer(64)
    lib().or_java_format2(float(x), buf, 64)
    return buf.value.decode()
