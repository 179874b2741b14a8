"""The host graph builder of tests/assembler_host.py on the CPU: Assembler.buildGraph's
kGraph / altGraph maps (S/Assembler.scala:132-154) built from the tally's edge
records, with a test-only stand-in whose kmer_tally returns the oracle's edges.
Each K-mer is visited once in buildGraph, so its kGraph entry is the called
base's successor and altGraph holds the alternate base's when the call is not
homozygous."""
from oracle import oracle
from pilon_gb300 import _abi
from tests.assembler_host import Assembler, kmer_string
from pilon_gb300.reads import build_store


class _OracleTally:
    def __init__(self, reads):
        self.reads = reads

    def kmer_tally(self, windows, K, params, min_depth=5):
        return oracle.kmer_tally(self.reads, params, windows, K, min_depth)


def _read(pos, seq):
    return dict(pos=pos, cigar=[(len(seq), "M")], seq=seq, qual=[30] * len(seq), mapq=20)


def test_graphs_of_two_windows():
    """Window 0: five copies of ACGTTACG, K = 3 (the hand case of the tally):
    forward ACG->T, CGT->T, GTT->A, TTA->C, TAC->G; reverse complement CGTAACGT:
    CGT->A, GTA->A, TAA->C, AAC->G, ACG->T.  CGT ties 5 T against 5 A, so the call
    is A (lower index) and not homozygous: kGraph CGT -> GTA, altGraph CGT -> GTT.
    Window 1: four copies (depth 4 < 5 except ACG and CGT at 8)."""
    st = build_store([_read(10, "ACGTTACG")] * 9)
    a = Assembler(_OracleTally(st), K=3)
    assert a.add_reads(0, 5) == 0 and a.add_reads(5, 9) == 1
    (k0, alt0), (k1, alt1) = a.build_graph(_abi.default_params())
    assert k0 == {"ACG": "CGT", "CGT": "GTA", "GTT": "TTA", "TTA": "TAC", "TAC": "ACG", "GTA": "TAA",
                  "TAA": "AAC", "AAC": "ACG"}
    assert alt0 == {"CGT": "GTT"}
    assert k1 == {"ACG": "CGT", "CGT": "GTA"} and alt1 == {"CGT": "GTT"}


def test_kmer_string_of_packed_keys():
    """4-bit BAM codes, first character in the top nibble of key_hi, the 17th
    onwards in key_lo."""
    s = "ACGTNACGTTGCAACGTA"  # 18 characters
    code = {c: i for i, c in enumerate("=ACMGRSVTWYHKDBN")}
    hi = lo = 0
    for j, ch in enumerate(s):
        if j < 16:
            hi |= code[ch] << (60 - 4 * j)
        else:
            lo |= code[ch] << (60 - 4 * (j - 16))
    assert kmer_string(hi, lo, len(s)) == s
