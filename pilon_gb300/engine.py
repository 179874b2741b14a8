"""ctypes binding of libpilon_gb300.so, the GB300 engine behind the C ABI of
include/pilon_gb300.h.  A JVM host would make the same calls through JNI or
the Java foreign-function API.

There is no CPU fallback: if the engine library is missing or no CUDA device
is present, every call raises.
"""
import ctypes as C
import os

import numpy as np

from . import _abi
from .build import ENGINE

_LIB = None


class EngineError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{_abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def lib():
    """Loads the engine library; raises if it was not built."""
    global _LIB
    if _LIB is None:
        path = os.environ.get("PILON_GB300_ENGINE", ENGINE)  # an alternative build of the same ABI
        if not os.path.exists(path):
            raise EngineError(-1, f"engine library {path} is missing; run pilon_gb300.build.build()")
        L = C.CDLL(path)
        vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
        sig = {
            "pg_open": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
            "pg_close": (None, [vp]),
            "pg_last_error": (C.c_char_p, [vp]),
            "pg_default_params": (None, [C.POINTER(_abi.pg_params)]),
            "pg_version": (C.c_char_p, []),
            "pg_set_reference": (C.c_int, [vp, i32, vp, vp]),
            "pg_set_reads": (C.c_int, [vp, C.POINTER(_abi.pg_reads)]),
            "pg_set_reads_device": (C.c_int, [vp, C.POINTER(_abi.pg_reads)]),
            "pg_set_reads_packed": (C.c_int, [vp, C.POINTER(_abi.pg_reads)]),
            "pg_pileup_regions": (C.c_int, [vp, vp, i32, C.POINTER(_abi.pg_params), i32]),
            "pg_fetch_stats": (C.c_int, [vp, i32, C.POINTER(_abi.pg_region_stats)]),
            "pg_fetch_region": (C.c_int, [vp, i32, C.POINTER(_abi.pg_region_out)]),
            "pg_fetch_all": (C.c_int, [vp, C.POINTER(_abi.pg_region_out)]),
            "pg_set_tuning": (C.c_int, [vp, i32, i32, i32]),
            "pg_kmer_tally": (C.c_int, [vp, vp, i32, i32, C.POINTER(_abi.pg_params), i32, vp, i64,
                                        C.POINTER(C.c_int64)]),
            "pg_kmer_tally_wide": (C.c_int, [vp, vp, i32, i32, C.POINTER(_abi.pg_params), i32, vp, i64,
                                             C.POINTER(C.c_int64)]),
            "pg_kmer_tally_breaks_wide": (C.c_int, [vp, i32, i32, i32, C.POINTER(_abi.pg_params), i32, vp, i64,
                                                    C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
            "pg_last_kernel_ms": (C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                            C.POINTER(C.c_int32)]),
            "pg_sync": (C.c_int, [vp]),
            "pg_graph_replays": (C.c_int, [vp, C.POINTER(C.c_int32)]),
            "pg_last_tally_stats": (C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                              C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
            "pg_default_serve_config": (None, [C.POINTER(_abi.pg_serve_config)]),
            "pg_serve_open": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(_abi.pg_serve_config),
                                        C.POINTER(_abi.pg_params), i32, vp, vp, vp, C.POINTER(_abi.pg_reads)]),
            "pg_serve_submit": (C.c_int, [vp, C.POINTER(_abi.pg_request), C.POINTER(C.c_uint64)]),
            "pg_serve_poll": (C.c_int, [vp, C.c_uint64, i32, C.POINTER(_abi.pg_result)]),
            "pg_serve_release": (C.c_int, [vp, C.c_uint64]),
            "pg_serve_stats": (C.c_int, [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
            "pg_serve_error": (C.c_char_p, [vp]),
            "pg_serve_close": (None, [vp]),
            "pg_format_vcf": (C.c_int, [vp, i32, C.c_char_p, i32, i32, i32, vp, i64, C.POINTER(C.c_int64)]),
            "pg_find_breaks": (C.c_int, [vp, i32, vp, i64, C.POINTER(C.c_int64)]),
            "pg_find_duplications": (C.c_int, [vp, vp, i64, C.POINTER(C.c_int64)]),
            "pg_fetch_changes": (C.c_int, [vp, vp, i64, C.POINTER(C.c_int64), vp, i64, C.POINTER(C.c_int64)]),
            "pg_kmer_tally_breaks": (C.c_int, [vp, i32, i32, i32, C.POINTER(_abi.pg_params), i32, vp, i64,
                                               C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
            "pg_kmer_tally_reads": (C.c_int, [vp, vp, i64, vp, i32, i32, C.POINTER(_abi.pg_params), i32, vp, i64,
                                              C.POINTER(C.c_int64)]),
            "pg_reassemble": (C.c_int, [vp, i64, i32, vp, i32, i32, vp, vp, i64, C.POINTER(C.c_int64)]),
            "pg_region_fixes": (C.c_int, [vp, i64, vp, i64, vp, i64, i32, i32, C.POINTER(_abi.pg_fix_options), vp,
                                          vp, i64, C.POINTER(C.c_int64), vp, i64, C.POINTER(C.c_int64), vp, vp,
                                          i64, C.POINTER(C.c_int64)]),
            "pg_changes_lines": (C.c_int, [vp, i64, vp, i64, C.c_char_p, C.c_char_p, i64, vp, i64,
                                           C.POINTER(C.c_int64)]),
            "pg_scan_reads": (C.c_int, [C.POINTER(_abi.pg_reads), C.POINTER(_abi.pg_params), i32, i32, i32, vp, vp,
                                        i64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
            "pg_mark_deleted": (C.c_int, [vp, i32, i32, i32]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


class RegionArrays:
    """One region's pileup records and calls on the host (pg_region_out)."""
    I32 = ["mq_sum", "q_sum", "phys_cov", "insert_size", "bad_pair", "deletions", "del_qual", "insertions",
           "ins_qual", "clips", "indel_len", "ins_str"]

    def __init__(self, size):
        self.size = size
        self.count = np.empty(4 * size, np.int32)
        self.qual_sum = np.empty(4 * size, np.int64)
        for f in self.I32:
            setattr(self, f, np.empty(size, np.int32))
        self.call = np.empty(size, np.uint32)
        self.score = np.empty(size, np.int64)
        self.ins_chars = np.zeros(0, np.uint8)
        self.stats = _abi.pg_region_stats()

    def out_struct(self, ins_cap):
        o = _abi.pg_region_out()
        ptr = lambda a: a.ctypes.data if a is not None else None
        o.count = ptr(self.count)
        o.qual_sum = ptr(self.qual_sum)
        for f in self.I32:
            setattr(o, f, ptr(getattr(self, f)))
        o.call = ptr(self.call)
        o.score = ptr(self.score)
        if self.ins_chars.size < ins_cap:
            self.ins_chars = np.zeros(ins_cap, np.uint8)
        o.ins_chars = self.ins_chars.ctypes.data if self.ins_chars.size else None
        o.ins_chars_cap = self.ins_chars.size
        return o

    def insertion(self, i):
        off = int(self.ins_str[i])
        if off < 0:
            return ""
        return self.ins_chars[off:off + int(self.indel_len[i])].tobytes().decode()


class Engine:
    """One engine context on one CUDA device (pg_open ... pg_close)."""

    def __init__(self, device=0):
        self.L = lib()
        self.h = C.c_void_p()
        st = self.L.pg_open(C.byref(self.h), device)
        if st != 0:
            msg = self.L.pg_last_error(self.h).decode() if self.h else "pg_open failed"
            if self.h:
                self.L.pg_close(self.h)
            self.h = None
            raise EngineError(st, msg)
        self._keep = []

    def close(self):
        if self.h:
            self.L.pg_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != 0:
            raise EngineError(st, self.L.pg_last_error(self.h).decode())

    def set_reference(self, contigs):
        arrs = [np.ascontiguousarray(c, np.uint8) for c in contigs]
        lens = np.array([a.size for a in arrs], np.int64)
        ptrs = (C.c_void_p * max(1, len(arrs)))(*[a.ctypes.data for a in arrs])
        self._check(self.L.pg_set_reference(self.h, len(arrs), lens.ctypes.data, C.cast(ptrs, C.c_void_p)))
        self.contig_lens = lens

    def set_reads(self, reads, packed=False):
        """pg_set_reads, or pg_set_reads_packed (packed=True: the store's offsets
        and alignment ends are derived on the device and not uploaded)."""
        ab = reads.to_abi()
        fn = self.L.pg_set_reads_packed if packed else self.L.pg_set_reads
        self._check(fn(self.h, C.byref(ab)))
        self.n_reads = reads.n_reads

    def set_tuning(self, tile_width=0, warps=0, variant=-1):
        self._check(self.L.pg_set_tuning(self.h, tile_width, warps, variant))

    _REGION_DT = np.dtype([("contig", "<i4"), ("start", "<i4"), ("stop", "<i4"), ("pad_", "<i4"),
                           ("read_begin", "<i8"), ("read_end", "<i8")])

    def _region_array(self, regions):
        """The pg_region array of a region list; the last one is kept, so a host
        calling again with the same regions (a serving loop, a benchmark) does
        not build it again."""
        key = tuple(map(tuple, regions))
        cached = getattr(self, "_regions_cache", None)
        if cached is not None and cached[0] == key:
            return cached[1]
        arr = np.zeros(max(1, len(regions)), self._REGION_DT)
        if len(regions):
            a = np.asarray(regions, dtype=np.int64).reshape(len(regions), 5)
            arr["contig"][:len(regions)] = a[:, 0]
            arr["start"][:len(regions)] = a[:, 1]
            arr["stop"][:len(regions)] = a[:, 2]
            arr["read_begin"][:len(regions)] = a[:, 3]
            arr["read_end"][:len(regions)] = a[:, 4]
        self._regions_cache = (key, arr)
        return arr

    def pileup_regions(self, regions, params, batched=True):
        """regions: list of (contig, start, stop, read_begin, read_end)."""
        arr = self._region_array(regions)
        self._check(self.L.pg_pileup_regions(self.h, C.c_void_p(arr.ctypes.data), len(regions), C.byref(params),
                                             int(batched)))
        self.regions = list(regions)

    def stats(self, r):
        st = _abi.pg_region_stats()
        self._check(self.L.pg_fetch_stats(self.h, r, C.byref(st)))
        return st

    def fetch(self, r, out=None):
        c, s, e, _, _ = self.regions[r]
        size = e - s + 1
        out = out or RegionArrays(size)
        o = out.out_struct(0)
        o.ins_chars = None
        self._check(self.L.pg_fetch_region(self.h, r, C.byref(o)))
        pool = int(o.ins_chars_cap)
        if pool:
            o2 = _abi.pg_region_out()
            out.ins_chars = np.zeros(pool, np.uint8)
            o2.ins_chars = out.ins_chars.ctypes.data
            o2.ins_chars_cap = pool
            self._check(self.L.pg_fetch_region(self.h, r, C.byref(o2)))
        out.stats = self.stats(r)
        return out

    def fetch_all(self, out):
        """pg_fetch_all into `out` (RegionArrays sized for every position of the
        last call, regions one after another); insertion characters not read."""
        o = out.out_struct(0)
        o.ins_chars = None
        self._check(self.L.pg_fetch_all(self.h, C.byref(o)))
        return out

    def kmer_tally(self, windows, K, params, min_depth=5, cap=None, wide=None):
        """Edges of every window (pg_kmer_tally, K <= 31, or pg_kmer_tally_wide,
        K <= 63: the wide form, four key words, when wide or K > 31)."""
        wide = K > 31 if wide is None else wide
        wins = (_abi.pg_window * max(1, len(windows)))(*[_abi.pg_window(a, b) for a, b in windows])
        fn = self.L.pg_kmer_tally_wide if wide else self.L.pg_kmer_tally
        dt = _abi.kmer_edge_wide_dtype() if wide else _abi.kmer_edge_dtype()
        # start from the last call's edge count, so a repeated call runs once
        cap = cap or getattr(self, "_kmer_cap", 1 << 20)
        while True:
            edges = np.zeros(cap, dt)
            n = C.c_int64()
            self._check(fn(self.h, C.cast(wins, C.c_void_p), len(windows), K, C.byref(params), min_depth,
                           edges.ctypes.data, cap, C.byref(n)))
            if n.value <= cap:
                self._kmer_cap = max(cap, int(n.value))
                return edges[:n.value]
            cap = int(n.value)

    def kmer_tally_reads(self, read_lists, K, params, min_depth=5, cap=None):
        """pg_kmer_tally_reads: edges (pg_kmer_edge_wide records) of one window
        per list of read indices."""
        lens = np.array([len(x) for x in read_lists], np.int64)
        bounds = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
        reads = (np.concatenate([np.asarray(x, np.int64) for x in read_lists]).astype(np.int64)
                 if len(read_lists) else np.zeros(0, np.int64))
        wins = np.stack([bounds[:-1], bounds[1:]], axis=1).astype(np.int64) if len(read_lists) else \
            np.zeros((0, 2), np.int64)
        wins = np.ascontiguousarray(wins)
        reads = np.ascontiguousarray(reads)
        dt = _abi.kmer_edge_wide_dtype()
        cap = cap or getattr(self, "_kmer_cap", 1 << 20)
        while True:
            edges = np.zeros(cap, dt)
            n = C.c_int64()
            self._check(self.L.pg_kmer_tally_reads(self.h, reads.ctypes.data, reads.size, wins.ctypes.data,
                                                   len(read_lists), K, C.byref(params), min_depth,
                                                   edges.ctypes.data, cap, C.byref(n)))
            if n.value <= cap:
                self._kmer_cap = max(cap, int(n.value))
                return edges[:n.value]
            cap = int(n.value)

    def mark_deleted(self, r, first_locus, count):
        """pg_mark_deleted: loci of region r that a reassembly fix replaces."""
        self._check(self.L.pg_mark_deleted(self.h, r, first_locus, count))

    def format_vcf(self, r, name, diploid=False, vcf_qe=False, variants_only=False):
        """The region's VCF records as bytes (pg_format_vcf)."""
        n = C.c_int64()
        args = (self.h, r, name.encode(), int(diploid), int(vcf_qe), int(variants_only))
        st = self.L.pg_format_vcf(*args, None, 0, C.byref(n))
        if st not in (0, _abi.PG_ERR_LIMIT):
            self._check(st)
        buf = np.empty(max(int(n.value), 1), np.uint8)
        self._check(self.L.pg_format_vcf(*args, buf.ctypes.data, buf.size, C.byref(n)))
        return buf[:n.value].tobytes()

    def find_breaks(self, min_min_depth=5):
        """pg_find_breaks: break candidates of every region of the last
        pileup_regions call, as {region: [(start, stop), ...]}."""
        n = C.c_int64()
        self._check(self.L.pg_find_breaks(self.h, min_min_depth, None, 0, C.byref(n)))
        buf = (_abi.pg_break * max(1, n.value))()
        self._check(self.L.pg_find_breaks(self.h, min_min_depth, C.cast(buf, C.c_void_p), n.value, C.byref(n)))
        out = {}
        for k in range(n.value):
            b = buf[k]
            out.setdefault(int(b.region), []).append((int(b.start), int(b.stop)))
        return out

    def fetch_changes(self, cap=None, ins_cap=None):
        """pg_fetch_changes: (changes as a pg_change array ordered by region and
        locus, insertion characters) of the last pileup_regions call."""
        cap = cap or getattr(self, "_chg_cap", 1 << 16)
        ins_cap = ins_cap or getattr(self, "_ins_cap", 1 << 16)
        while True:
            out = np.zeros(cap, _abi.change_dtype())
            chars = np.zeros(ins_cap, np.uint8)
            n, ni = C.c_int64(), C.c_int64()
            self._check(self.L.pg_fetch_changes(self.h, out.ctypes.data, cap, C.byref(n), chars.ctypes.data, ins_cap,
                                                C.byref(ni)))
            if n.value <= cap and ni.value <= ins_cap:
                self._chg_cap, self._ins_cap = cap, ins_cap
                return out[:n.value], chars[:ni.value].tobytes()
            cap, ins_cap = max(cap, int(n.value)), max(ins_cap, int(ni.value))

    def find_duplications(self):
        """pg_find_duplications: the <DUP> regions (duplicationEvents) of every
        region of the last pileup_regions call, as {region: [(start, stop), ...]}."""
        n = C.c_int64()
        self._check(self.L.pg_find_duplications(self.h, None, 0, C.byref(n)))
        buf = (_abi.pg_break * max(1, n.value))()
        self._check(self.L.pg_find_duplications(self.h, C.cast(buf, C.c_void_p), n.value, C.byref(n)))
        out = {}
        for k in range(n.value):
            b = buf[k]
            out.setdefault(int(b.region), []).append((int(b.start), int(b.stop)))
        return out

    def kmer_tally_breaks(self, K, params, radius=500, min_depth=5, cap=None, wide=None):
        """pg_kmer_tally_breaks (K <= 31) or pg_kmer_tally_breaks_wide (K <= 63):
        the K-mer tally over one device-built window per break candidate;
        returns (number of windows, edges)."""
        wide = K > 31 if wide is None else wide
        fn = self.L.pg_kmer_tally_breaks_wide if wide else self.L.pg_kmer_tally_breaks
        dt = _abi.kmer_edge_wide_dtype() if wide else _abi.kmer_edge_dtype()
        cap = cap or getattr(self, "_kmer_cap", 1 << 20)
        while True:
            edges = np.zeros(cap, dt)
            nw, n = C.c_int64(), C.c_int64()
            self._check(fn(self.h, params.min_min_depth, radius, K, C.byref(params), min_depth, edges.ctypes.data,
                           cap, C.byref(nw), C.byref(n)))
            if n.value <= cap:
                self._kmer_cap = max(cap, int(n.value))
                return int(nw.value), edges[:n.value]
            cap = int(n.value)

    def set_reads_device(self, dev_reads, n_reads):
        """pg_set_reads_device: a read store already in device memory (pg_reads
        with device pointers), shared by several contexts."""
        self._check(self.L.pg_set_reads_device(self.h, C.byref(dev_reads)))
        self.n_reads = n_reads

    def last_kernel_ms(self):
        w, t, n = C.c_double(), C.c_double(), C.c_int32()
        self._check(self.L.pg_last_kernel_ms(self.h, C.byref(w), C.byref(t), C.byref(n)))
        return w.value, t.value, n.value

    def sync(self):
        self._check(self.L.pg_sync(self.h))

    def last_tally_stats(self):
        """pg_last_tally_stats: (kernel ms, K-mer events, distinct K-mers, largest
        batch's table bytes, batches) of the last K-mer tally."""
        ms, ev, dk, tb, nb = C.c_double(), C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32()
        self._check(self.L.pg_last_tally_stats(self.h, C.byref(ms), C.byref(ev), C.byref(dk), C.byref(tb),
                                               C.byref(nb)))
        return ms.value, ev.value, dk.value, tb.value, nb.value

    def graph_replays(self):
        """pg_graph_replays: calls of this context that replayed a recorded graph."""
        n = C.c_int32()
        self._check(self.L.pg_graph_replays(self.h, C.byref(n)))
        return n.value


def region_fixes(changes, chars, contig, start, stop, fix_snps=True, fix_indels=True, iupac=False,
                 long_read=False, excluded=None):
    """pg_region_fixes on the host: one region's pg_change records (a slice of
    fetch_changes) and the insertion characters -> (fixes as a pg_fix array,
    snp list then small list, each last change first; their strings; the bases
    after the SNP fixes; the bases after the small fixes too)."""
    L = lib()
    ch = np.ascontiguousarray(changes, _abi.change_dtype())
    ins = np.frombuffer(chars, np.uint8) if len(chars) else np.zeros(1, np.uint8)
    contig = np.ascontiguousarray(contig, np.uint8)
    ex = None if excluded is None else np.ascontiguousarray(excluded, np.uint8)
    opts = _abi.pg_fix_options(int(fix_snps), int(fix_indels), int(iupac), int(long_read))
    size = stop - start + 1
    nf, tl, bl = C.c_int64(), C.c_int64(), C.c_int64()
    fcap, tcap, bcap = max(1, ch.size), max(16, 4 * ch.size), size + 64
    while True:
        fixes = np.zeros(fcap, _abi.fix_dtype())
        text = np.zeros(tcap, np.uint8)
        snp = np.zeros(size, np.uint8)
        out = np.zeros(bcap, np.uint8)
        st = L.pg_region_fixes(ch.ctypes.data if ch.size else None, ch.size, ins.ctypes.data, len(chars),
                               contig.ctypes.data, contig.size, start, stop, C.byref(opts),
                               ex.ctypes.data if ex is not None else None, fixes.ctypes.data, fcap, C.byref(nf),
                               text.ctypes.data, tcap, C.byref(tl), snp.ctypes.data, out.ctypes.data, bcap,
                               C.byref(bl))
        if st == _abi.PG_ERR_LIMIT and (nf.value > fcap or tl.value > tcap or bl.value > bcap):
            fcap, tcap, bcap = max(fcap, nf.value), max(tcap, tl.value), max(bcap, bl.value)
            continue
        if st:
            raise EngineError(st, "pg_region_fixes: bad changes for the region")
        return fixes[:nf.value], text[:tl.value].tobytes(), snp.tobytes(), out[:bl.value].tobytes()


def changes_lines(fixes, text, name, new_name, offset):
    """pg_changes_lines on the host: the changes file's lines of one region
    from its fixes (pg_fix array, snp ++ small ++ big), as bytes."""
    L = lib()
    fx = np.ascontiguousarray(fixes, _abi.fix_dtype())
    tb = np.frombuffer(text, np.uint8) if len(text) else np.zeros(1, np.uint8)
    cap = max(256, 64 * fx.size)
    n = C.c_int64()
    while True:
        out = np.zeros(cap, np.uint8)
        st = L.pg_changes_lines(fx.ctypes.data if fx.size else None, fx.size, tb.ctypes.data, len(text),
                                name.encode(), new_name.encode(), offset, out.ctypes.data, cap, C.byref(n))
        if st == _abi.PG_ERR_LIMIT and n.value > cap:
            cap = n.value
            continue
        if st:
            raise EngineError(st, "pg_changes_lines: bad fixes")
        return out[:n.value].tobytes()


def scan_reads(reads, params, n_contigs, huge, strays=True, threads=0):
    """pg_scan_reads on the host: (the 9 insert statistics: FR, RF, unpaired
    count, sum, sumSq; the first-of-pair stray-mate read indices; the
    second-of-pair ones), the index arrays empty when strays is False."""
    L = lib()
    ab = reads.to_abi()
    stats = np.zeros(9, np.int64)
    nf, ns = C.c_int64(), C.c_int64()
    cap = max(1024, reads.n_reads // 64) if strays else 0
    while True:
        out = np.zeros(max(cap, 1), np.int64)
        st = L.pg_scan_reads(C.byref(ab), C.byref(params), n_contigs, huge, threads, stats.ctypes.data,
                             out.ctypes.data, cap, C.byref(nf), C.byref(ns))
        if st == _abi.PG_ERR_LIMIT and strays:
            cap = nf.value + ns.value
            continue
        if st and not (st == _abi.PG_ERR_LIMIT and not strays):
            raise EngineError(st, "pg_scan_reads: bad arguments")
        if not strays:
            return stats, np.zeros(0, np.int64), np.zeros(0, np.int64)
        return stats, out[:nf.value].copy(), out[nf.value:nf.value + ns.value].copy()


def reassemble(edges, K, jobs, threads=0):
    """pg_reassemble on the host: jobs are dicts (window, is_gap, region_start,
    region_stop, break_start, break_stop, break_radius, bases, orig), the
    region's bases as contiguous uint8 arrays (shared by the jobs of one
    region); returns one (start, was, patch, status, loop_len) per job, start 0
    when there is no solution."""
    L = lib()
    n = len(jobs)
    arr = (_abi.pg_reassembly * max(1, n))()
    for k, j in enumerate(jobs):
        b, o = j["bases"], j["orig"]
        for x in (b, o):
            if not (isinstance(x, np.ndarray) and x.dtype == np.uint8 and x.flags.c_contiguous and
                    x.size == j["region_stop"] + 1 - j["region_start"]):
                raise ValueError("job bases must be contiguous uint8 arrays of the region's size")
        arr[k] = _abi.pg_reassembly(j["window"], int(j["is_gap"]), j["region_start"], j["region_stop"],
                                    j["break_start"], j["break_stop"], j["break_radius"],
                                    int(j.get("fix_breaks", 0)), int(j.get("gap_margin", 100000)),
                                    int(j.get("min_gap", 10)), b.ctypes.data, o.ctypes.data)
    fixes = (_abi.pg_reassembly_fix * max(1, n))()
    edges = np.ascontiguousarray(edges)
    cap = 1 << 16
    while True:
        text = np.zeros(cap, np.uint8)
        tl = C.c_int64()
        st = L.pg_reassemble(edges.ctypes.data if edges.size else None, edges.size, K, C.cast(arr, C.c_void_p), n,
                             threads, C.cast(fixes, C.c_void_p), text.ctypes.data, cap, C.byref(tl))
        if st == _abi.PG_ERR_LIMIT and tl.value > cap:
            cap = int(tl.value)
            continue
        if st:
            raise EngineError(st, "pg_reassemble: bad arguments" if st == _abi.PG_ERR_ARG
                              else "pg_reassemble: host memory or threads exhausted")
        break
    t = text.tobytes()
    out = []
    for k in range(n):
        f = fixes[k]
        out.append((int(f.start), t[f.was_off:f.was_off + f.was_len].decode(),
                    t[f.patch_off:f.patch_off + f.patch_len].decode(), int(f.status), int(f.loop_len)))
    return out
