"""BAM input and output for the packed read store.

read_bam is the host side of BamFile's input (S/BamFile.scala:117-126, which
htsjdk decodes): libpg_bam.so inflates the BGZF blocks of the file on native
threads, each straight into its place in one buffer (its own raw-DEFLATE
decoder), and splits the record stream into the structure-of-arrays store of
the C ABI, keeping BAM's CIGAR words, 4-bit bases and qualities as they are.  write_bam writes a
store as a coordinate-sorted BAM (read names r<index>, no tags), for tests and
the benchmark.
"""
import ctypes as C
import mmap
import os
import struct
import zlib
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from .reads import ReadStore

BGZF_EOF = bytes.fromhex("1f8b08040000000000ff0600424302001b0003000000000000000000")
_BLOCK = 65280  # uncompressed bytes per BGZF block
_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        from .build import BAMLIB, build
        if not os.path.exists(BAMLIB):
            build()
        L = C.CDLL(BAMLIB)
        vp, i64 = C.c_void_p, C.c_int64
        L.bam_index.restype = i64
        L.bam_index.argtypes = [vp, i64, vp, i64, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]
        L.bam_fill.restype = i64
        L.bam_fill.argtypes = [vp, vp, i64] + [vp] * 15 + [C.c_int32]
        L.bam_encoded_size.restype = i64
        L.bam_encoded_size.argtypes = [i64, vp, vp, vp]
        L.bam_encode.restype = i64
        L.bam_encode.argtypes = [i64] + [vp] * 17
        L.bam_name_ids.restype = i64
        L.bam_name_ids.argtypes = [vp, vp, i64, vp]
        L.bgzf_scan.restype = i64
        L.bgzf_scan.argtypes = [vp, i64, vp, vp, vp, i64, C.POINTER(i64), C.POINTER(C.c_int32)]
        L.bgzf_inflate_blocks.restype = i64
        L.bgzf_inflate_blocks.argtypes = [vp, i64, vp, vp, vp, vp, vp, C.c_int32]
        _LIB = L
    return _LIB


def _threads(threads):
    return threads or min(32, os.cpu_count() or 1)


def _bgzf_block(data):
    c = zlib.compressobj(1, zlib.DEFLATED, -15)
    cdata = c.compress(data) + c.flush()
    bsize = 18 + len(cdata) + 8 - 1
    head = struct.pack("<BBBBIBBHBBHH", 0x1F, 0x8B, 8, 4, 0, 0, 0xFF, 6, 66, 67, 2, bsize)
    return head + cdata + struct.pack("<II", zlib.crc32(data) & 0xFFFFFFFF, len(data))


def write_bam(path, names, lengths, reads, threads=None):
    """Writes `reads` (a ReadStore sorted by reference and position) as BAM."""
    text = "@HD\tVN:1.6\tSO:coordinate\n" + "".join(f"@SQ\tSN:{n}\tLN:{l}\n" for n, l in zip(names, lengths))
    tb = text.encode()
    hdr = bytearray(b"BAM\x01" + struct.pack("<i", len(tb)) + tb + struct.pack("<i", len(names)))
    for n, l in zip(names, lengths):
        nb = n.encode() + b"\0"
        hdr += struct.pack("<i", len(nb)) + nb + struct.pack("<i", int(l))
    r = reads
    L = _lib()
    n = r.n_reads
    nid = None if r.name_id is None else np.ascontiguousarray(r.name_id, np.int64)
    nptr = None if nid is None else nid.ctypes.data
    size = L.bam_encoded_size(n, r.n_cigar.ctypes.data, r.l_seq.ctypes.data, nptr)
    recs = np.empty(max(size, 1), np.uint8)
    L.bam_encode(n, r.pos.ctypes.data, r.tlen.ctypes.data, r.ref_id.ctypes.data, r.mate_ref_id.ctypes.data,
                 r.l_seq.ctypes.data, r.flag.ctypes.data, r.n_cigar.ctypes.data, r.mapq.ctypes.data,
                 r.seq.ctypes.data, r.qual.ctypes.data, r.cigar_off.ctypes.data, r.seq_off.ctypes.data,
                 r.qual_off.ctypes.data, r.cigar.ctypes.data, None, nptr, recs.ctypes.data)
    payload = memoryview(bytes(hdr) + recs[:size].tobytes())
    chunks = [payload[k:k + _BLOCK] for k in range(0, len(payload), _BLOCK)]
    with ThreadPoolExecutor(_threads(threads)) as ex:
        blocks = list(ex.map(lambda ch: _bgzf_block(bytes(ch)), chunks))
    with open(path, "wb") as f:
        for b in blocks:
            f.write(b)
        f.write(BGZF_EOF)


_SCAN_ERRORS = {1: "is not a BGZF block", 2: "is truncated", 3: "has no BC field",
                4: "claims more than 65536 uncompressed bytes", 5: "exceeds the block count bound"}


def _block_table(raw):
    """(cdata offsets, cdata ends, uncompressed sizes) of every BGZF block, as
    int64 arrays, from the native scan of the gzip member headers."""
    n = len(raw)
    inp = np.frombuffer(raw, np.uint8) if n else np.zeros(1, np.uint8)
    cap = n // 28 + 1
    src, end, size = (np.empty(cap, np.int64) for _ in range(3))
    err_off, err_kind = C.c_int64(), C.c_int32()
    k = _lib().bgzf_scan(inp.ctypes.data, n, src.ctypes.data, end.ctypes.data, size.ctypes.data, cap,
                         C.byref(err_off), C.byref(err_kind))
    del inp  # a view of a mapped file must not outlive this call (the caller closes the map)
    if k < 0:
        raise ValueError(f"BGZF block at byte {err_off.value} {_SCAN_ERRORS.get(err_kind.value, 'is damaged')}")
    return src[:k], end[:k], size[:k]


def _blocks(raw):
    """(cdata offset, cdata end, uncompressed size) of every BGZF block."""
    return [tuple(int(x) for x in t) for t in zip(*_block_table(raw))]


def inflate_blocks(raw, blocks, threads=None):
    """The uncompressed bytes of the BGZF blocks (cdata start, cdata end,
    uncompressed size) of `raw`, one after another; `blocks` is a list of such
    triples or the three arrays of _block_table."""
    if isinstance(blocks, tuple) and len(blocks) == 3 and isinstance(blocks[0], np.ndarray):
        src, end, sizes = (np.ascontiguousarray(b, np.int64) for b in blocks)
        n = src.size
    else:
        n = len(blocks)
        src = np.array([b[0] for b in blocks], np.int64).reshape(n)
        end = np.array([b[1] for b in blocks], np.int64).reshape(n)
        sizes = np.array([b[2] for b in blocks], np.int64).reshape(n)
    starts = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    data = np.empty(max(int(starts[-1]), 1), np.uint8)
    inp = np.frombuffer(raw, np.uint8) if len(raw) else np.zeros(1, np.uint8)
    rc = _lib().bgzf_inflate_blocks(inp.ctypes.data, n, src.ctypes.data, end.ctypes.data, starts.ctypes.data,
                                    sizes.ctypes.data, data.ctypes.data, _threads(threads))
    del inp  # no view of a mapped file may outlive this call
    if rc < 0:
        raise ValueError(f"BGZF block {-rc - 1}: damaged DEFLATE data or wrong uncompressed size")
    return data[:int(starts[-1])]


def _header(view):
    """Reference names and lengths of the BAM header (magic, l_text, text,
    n_ref, then l_name, name with its NUL, l_ref per reference) and the offset
    of the first record."""
    n = len(view)

    def i32(at):
        if at < 0 or at + 4 > n:
            raise ValueError("BAM header is truncated")
        return struct.unpack_from("<i", view, at)[0]

    l_text = i32(4)
    if l_text < 0:
        raise ValueError("BAM header text length is negative")
    off = 8 + l_text
    n_ref = i32(off)
    if n_ref < 0:
        raise ValueError("BAM header reference count is negative")
    off += 4
    names, lengths = [], []
    for _ in range(n_ref):
        ln = i32(off)
        if ln < 1 or off + 8 + ln > n:
            raise ValueError("BAM header reference entry is damaged")
        names.append(bytes(view[off + 4:off + 4 + ln - 1]).decode("utf-8", "replace"))
        lengths.append(i32(off + 4 + ln))
        off += 8 + ln
    return names, lengths, off


def read_bam(path, threads=None, names=False):
    """Returns (reference names, reference lengths, ReadStore) of a BAM file.
    names=True also gives the store its read-name ids (store.name_id), which
    local reassembly pairs mates by (one more pass over the records)."""
    want_names = names
    with open(path, "rb") as f:
        # mapped, so that reading the file overlaps the threads' inflating
        raw = mmap.mmap(f.fileno(), 0, access=mmap.ACCESS_READ) if os.fstat(f.fileno()).st_size else b""
    try:
        data = inflate_blocks(raw, _block_table(raw), threads)
    finally:
        if isinstance(raw, mmap.mmap):
            raw.close()
    view = memoryview(data)
    if bytes(view[:4]) != b"BAM\x01":
        raise ValueError("not a BAM file")
    names, lengths, off = _header(view)
    L = _lib()
    recs = data[off:]
    nc, sb, qb = C.c_int64(), C.c_int64(), C.c_int64()
    # one walk of the record chain; a record takes at least 36 bytes, and the
    # pages of the unused tail of `starts` are never touched
    starts = np.empty(recs.size // 36 + 1, np.int64)
    n = L.bam_index(recs.ctypes.data, recs.size, starts.ctypes.data, starts.size, C.byref(nc), C.byref(sb),
                    C.byref(qb))
    if n < 0:
        raise ValueError(f"BAM record at stream byte {off - 1 - n} runs past the end of the file")
    st = ReadStore(pos=np.empty(n, np.int32), aend=np.empty(n, np.int32), flag=np.empty(n, np.uint16),
                   mapq=np.empty(n, np.uint8), tlen=np.empty(n, np.int32), ref_id=np.empty(n, np.int32),
                   mate_ref_id=np.empty(n, np.int32), cigar_off=np.empty(n, np.int64),
                   n_cigar=np.empty(n, np.uint16), cigar=np.empty(nc.value, np.uint32),
                   seq_off=np.empty(n, np.int64), l_seq=np.empty(n, np.int32), seq=np.empty(sb.value, np.uint8),
                   qual_off=np.empty(n, np.int64), qual=np.empty(qb.value, np.uint8))
    got = L.bam_fill(recs.ctypes.data, starts.ctypes.data, n, st.pos.ctypes.data, st.aend.ctypes.data,
                     st.tlen.ctypes.data, st.ref_id.ctypes.data, st.mate_ref_id.ctypes.data, st.l_seq.ctypes.data,
                     st.flag.ctypes.data, st.n_cigar.ctypes.data, st.mapq.ctypes.data, st.seq.ctypes.data,
                     st.qual.ctypes.data, st.cigar_off.ctypes.data, st.seq_off.ctypes.data, st.qual_off.ctypes.data,
                     st.cigar.ctypes.data, _threads(threads))
    if got != n:
        raise MemoryError("BAM record fill: host memory exhausted")
    if want_names:
        st.name_id = np.empty(n, np.int64)
        if L.bam_name_ids(recs.ctypes.data, starts.ctypes.data, n, st.name_id.ctypes.data) < 0:
            raise MemoryError("BAM read-name ids: host memory exhausted")
    return names, lengths, st
