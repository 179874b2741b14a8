"""Reference FASTA input (GenomeFile through htsjdk, S/GenomeFile.scala:30-42)
and its mapping onto the BAM's reference ids."""
import numpy as np
import pytest

from pilon_gb300.fasta import read_fasta, reference_for_bam


def test_names_cut_at_whitespace_raw_bytes_line_ends(tmp_path):
    f = tmp_path / "g.fa"
    f.write_bytes(b">chr1 first contig\r\nACGTacgt\r\nNNnn\r\n\n>chr2\tdesc\nGGCC\n>gi|123| x\nTT")
    names, contigs = read_fasta(str(f))
    assert names == ["chr1", "chr2", "gi|123|"]
    assert [c.tobytes() for c in contigs] == [b"ACGTacgtNNnn", b"GGCC", b"TT"]
    assert all(c.dtype == np.uint8 for c in contigs)


def test_empty_and_malformed(tmp_path):
    f = tmp_path / "e.fa"
    f.write_bytes(b"")
    assert read_fasta(str(f)) == ([], [])
    f.write_bytes(b"ACGT\n")
    with pytest.raises(ValueError):
        read_fasta(str(f))


def test_reference_for_bam_orders():
    """Contig i is the BAM's reference i; a FASTA contig the BAM lacks follows,
    a BAM reference the FASTA lacks is an empty placeholder, and the order to
    process is the FASTA's."""
    fn = ["b", "a", "c"]
    fc = [np.frombuffer(s, np.uint8) for s in (b"BBB", b"AA", b"C")]
    names, contigs, order = reference_for_bam(fn, fc, ["a", "b", "z"])
    assert names == ["a", "b", "z", "c"]
    assert [c.tobytes() for c in contigs] == [b"AA", b"BBB", b"", b"C"]
    assert order == [1, 0, 3]
    with pytest.raises(ValueError, match="no sequence"):
        reference_for_bam(["x"], [fc[0]], ["a", "b"])
