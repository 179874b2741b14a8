"""BAM input (BamFile's htsjdk decoding, S/BamFile.scala:117-126) into the read
store: round trips, the fields htsjdk derives, and damaged files."""
import gzip
import os
import struct
import tempfile

import numpy as np
import pytest

from pilon_gb300 import bam, synth
from pilon_gb300.reads import FIELDS


def test_round_trip_keeps_every_field(cfg1):
    ds = cfg1
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "reads.bam")
        bam.write_bam(path, ds.names, [c.size for c in ds.contigs], ds.reads, threads=4)
        # a BGZF file is a multi-member gzip file: the standard reader sees the same bytes
        assert gzip.open(path).read(4) == b"BAM\x01"
        names, lengths, st = bam.read_bam(path, threads=3)
    assert names == ds.names and lengths == [c.size for c in ds.contigs]
    for f in FIELDS:
        assert np.array_equal(getattr(st, f), getattr(ds.reads, f)), f


def test_many_contigs_and_absent_qualities():
    ds = synth.generate(3, scale=0.01)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "reads.bam")
        bam.write_bam(path, ds.names, [c.size for c in ds.contigs], ds.reads)
        names, lengths, st = bam.read_bam(path)
    assert len(names) == len(ds.contigs)
    for f in FIELDS:
        assert np.array_equal(getattr(st, f), getattr(ds.reads, f)), f


def test_alignment_end_of_unmapped_and_deletions(cfg1):
    """aend is htsjdk's getAlignmentEnd: start + reference length - 1, and 0
    for a read with the unmapped flag."""
    r = cfg1.reads.subset(np.arange(50))
    r.flag = r.flag.copy()
    r.flag[7] |= 0x4
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "u.bam")
        bam.write_bam(path, cfg1.names, [c.size for c in cfg1.contigs], r)
        _, _, st = bam.read_bam(path)
    assert st.aend[7] == 0
    keep = np.arange(50) != 7
    assert np.array_equal(st.aend[keep], r.aend[keep])


def test_truncated_file_is_an_error(cfg1):
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "reads.bam")
        bam.write_bam(path, cfg1.names, [c.size for c in cfg1.contigs], cfg1.reads.subset(np.arange(2000)))
        raw = open(path, "rb").read()
        bad = os.path.join(d, "bad.bam")
        open(bad, "wb").write(raw[: len(raw) // 2])
        with pytest.raises(ValueError):
            bam.read_bam(bad)
        # a record whose block_size runs past the stream, in an otherwise valid file
        small = os.path.join(d, "small.bam")
        bam.write_bam(small, cfg1.names, [c.size for c in cfg1.contigs], cfg1.reads.subset(np.arange(150)))
        raw = open(small, "rb").read()
        import zlib
        data = b"".join(zlib.decompress(raw[a:b], -15) for a, b, _ in bam._blocks(raw))
        cut = data[: len(data) - 10]
        assert len(cut) < 60000
        c = zlib.compressobj(1, zlib.DEFLATED, -15)
        cd = c.compress(cut) + c.flush()
        head = struct.pack("<BBBBIBBHBBHH", 0x1F, 0x8B, 8, 4, 0, 0, 0xFF, 6, 66, 67, 2, 18 + len(cd) + 8 - 1)
        open(bad, "wb").write(head + cd + struct.pack("<II", zlib.crc32(cut) & 0xFFFFFFFF, len(cut)) + bam.BGZF_EOF)
        with pytest.raises(ValueError):
            bam.read_bam(bad)


def _bam_of(payload):
    """A BGZF file holding `payload` in blocks of at most 60,000 bytes."""
    blocks = [bam._bgzf_block(payload[k:k + 60000]) for k in range(0, max(len(payload), 1), 60000)]
    return b"".join(blocks) + bam.BGZF_EOF


def _payload(cfg1, n=20):
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "r.bam")
        bam.write_bam(path, cfg1.names, [c.size for c in cfg1.contigs], cfg1.reads.subset(np.arange(n)))
        raw = open(path, "rb").read()
    import zlib
    return bytearray(b"".join(zlib.decompress(raw[a:b], -15) for a, b, _ in bam._blocks(raw)))


def _read(raw):
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "x.bam")
        open(path, "wb").write(raw)
        return bam.read_bam(path)


def test_damaged_headers_and_blocks_are_value_errors(cfg1):
    """Every damaged field a reader meets before the records raises ValueError:
    a block claiming more than 64 KiB, a header text or reference list that runs
    past the data, negative counts, an empty reference name entry."""
    good = _payload(cfg1)
    _read(_bam_of(bytes(good)))  # the rebuilt file itself reads
    blk = bytearray(_bam_of(bytes(good)))
    struct.pack_into("<I", blk, len(blk) - len(bam.BGZF_EOF) - 4, 70000)  # ISIZE of the last data block
    with pytest.raises(ValueError, match="uncompressed bytes"):
        _read(bytes(blk))
    l_text = struct.unpack_from("<i", good, 4)[0]
    for at, value in [(4, 1 << 30), (4, -5), (8 + l_text, -1), (8 + l_text, 1 << 20), (12 + l_text, 0),
                      (12 + l_text, 1 << 30)]:
        bad = bytearray(good)
        struct.pack_into("<i", bad, at, value)
        with pytest.raises(ValueError):
            _read(_bam_of(bytes(bad)))


def test_record_length_fields_are_checked(cfg1):
    """bam_index rejects a record whose l_seq, read-name length or CIGAR count
    does not fit its block_size (l_seq = 2^31 - 1 included); a position of
    2^31 - 1 reads back as htsjdk's wrapped Java int."""
    good = _payload(cfg1)
    l_text = struct.unpack_from("<i", good, 4)[0]
    off = 12 + l_text
    for _ in range(struct.unpack_from("<i", good, 8 + l_text)[0]):
        off += 8 + struct.unpack_from("<i", good, off)[0]
    rec = off + 4  # first record, after its block_size
    for field, fmt, value in [(16, "<i", 2 ** 31 - 1), (16, "<i", -1), (16, "<i", 10_000), (8, "<B", 255),
                              (12, "<H", 65535)]:
        bad = bytearray(good)
        struct.pack_into(fmt, bad, rec + field, value)
        with pytest.raises(ValueError, match="runs past"):
            _read(_bam_of(bytes(bad)))
    bad = bytearray(good)
    struct.pack_into("<i", bad, rec + 4, 2 ** 31 - 1)
    _, _, st = _read(_bam_of(bytes(bad)))
    assert st.pos[0] == -2 ** 31


def test_unplaced_tail_round_trip_and_plan(cfg1, tmp_path):
    """A coordinate-sorted BAM ending with unplaced reads (reference -1, BAM
    position -1): they read back with htsjdk's start 0 and end 0, and the region
    plan of the store leaves them out."""
    from pilon_gb300.reads import build_store, concat_stores
    from pilon_gb300.regions import plan_regions
    base = cfg1.reads.subset(np.arange(3000))
    rec = dict(pos=0, cigar=[], seq="ACGTNACGTT", qual=[20] * 10, flag=0x4, mapq=0, ref_id=-1, mate_ref_id=-1)
    store = concat_stores([base, build_store([rec] * 3)])
    lens = [c.size for c in cfg1.contigs]
    path = str(tmp_path / "u.bam")
    bam.write_bam(path, cfg1.names, lens, store)
    _, _, st = bam.read_bam(path)
    assert list(st.ref_id[-3:]) == [-1] * 3 and list(st.pos[-3:]) == [0] * 3 and list(st.aend[-3:]) == [0] * 3
    for f in FIELDS:
        assert np.array_equal(getattr(st, f), getattr(store, f)), f
    assert plan_regions(st, lens, 20000) == plan_regions(base, lens, 20000)
