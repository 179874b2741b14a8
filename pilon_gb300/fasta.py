"""Reference FASTA input, as GenomeFile loads it (S/GenomeFile.scala:30-42)
through htsjdk's ReferenceSequenceFileFactory: one contig per '>' record, the
name cut at the first whitespace of the header line, the bases kept as the
file's raw bytes (Pilon upper-cases them only where it compares a reference
base, S/GenomeRegion.scala:783-787; its indel shifts compare them raw).

The engine indexes contigs by the BAM's reference ids, while Pilon processes
and writes contigs in FASTA order; reference_for_bam maps one onto the other.
"""
import numpy as np


def read_fasta(path):
    """(names, contigs) of a FASTA file; contigs are uint8 arrays of the raw
    sequence bytes, line ends (LF or CRLF) removed."""
    with open(path, "rb") as f:
        data = f.read()
    names, contigs = [], []
    if not data.strip():
        return names, contigs
    if not data.lstrip().startswith(b">"):
        raise ValueError(f"{path}: a FASTA file starts with a '>' header line")
    for rec in data.lstrip()[1:].split(b"\n>"):
        head, _, body = rec.partition(b"\n")
        parts = head.split()
        if not parts:
            raise ValueError(f"{path}: a FASTA record without a name")
        names.append(parts[0].decode("utf-8", "replace"))
        contigs.append(np.frombuffer(body.translate(None, b"\r\n"), np.uint8).copy())
    return names, contigs


def reference_for_bam(fasta_names, fasta_contigs, bam_names):
    """The reference as the engine takes it for a BAM with references
    `bam_names`: (names, contigs, order).  Contig i is the BAM's reference i
    (an empty placeholder when the FASTA lacks it: no region is planned on it);
    the FASTA's contigs that the BAM lacks follow, so their regions get no reads,
    as a query of an unknown reference returns none.  `order` lists the FASTA's
    contigs in file order, the order Pilon processes and writes them.  Raises
    like BamFile.validateSeqs (S/BamFile.scala:77-79) when the BAM has none of
    the FASTA's contigs."""
    if len(set(fasta_names)) != len(fasta_names):
        raise ValueError("the FASTA names a contig twice")
    by_name = dict(zip(fasta_names, fasta_contigs))
    if not set(by_name) & set(bam_names):
        raise ValueError("the BAM has no sequence for any of " + ", ".join(fasta_names))
    names = list(bam_names)
    contigs = [by_name.get(n, np.zeros(0, np.uint8)) for n in bam_names]
    index = {n: i for i, n in enumerate(names)}
    for n in fasta_names:
        if n not in index:
            index[n] = len(names)
            names.append(n)
            contigs.append(by_name[n])
    return names, contigs, [index[n] for n in fasta_names]
