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
