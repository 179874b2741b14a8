"""CPU emulation of the pileup walk's four-bases-at-a-time decode.

The walk turns one word of BAM nibbles and one word of quality bytes into four
PileUp.add calls (S/PileUp.scala:75-84) without a branch per base: a prmt with
the nibbles as selectors looks each base code up in a table, a SWAR test checks
the quality bytes against minQual, and a second prmt builds each base's addend
qual + (1 << 20) for its row of counters.  This test restates that arithmetic
with the table constants read from the kernel source and checks it against
PileUp.add's rule -- the base is A/C/G/T and its quality, a signed byte, is at
least minQual -- for every nibble code, every quality byte and both parities of
the chunk's first read offset.
"""
import os
import re

import numpy as np
import pytest

SRC = os.path.join(os.path.dirname(__file__), "..", "pilon_gb300", "csrc", "pg_pileup.cu")
NIB = "=ACMGRSVTWYHKDBN"   # BAM 4-bit base codes


def _constants():
    s = open(SRC).read()
    m = re.search(r"kCodeLo = (0x[0-9a-fA-F]+)u, kCodeHi = (0x[0-9a-fA-F]+)u", s)
    c = re.search(r"comb = \(n0 & 1\) \? (0x[0-9a-fA-F]+)u : (0x[0-9a-fA-F]+)u", s)
    assert m and c, "decode constants not found in the kernel source"
    return int(m.group(1), 16), int(m.group(2), 16), int(c.group(2), 16), int(c.group(1), 16)


K_LO, K_HI, COMB_EVEN, COMB_ODD = _constants()


def prmt(a, b, s):
    """prmt.b32 default mode: byte k = byte (s >> 4k) & 7 of {b:a}, or its sign
    replicated when (s >> 4k) & 8."""
    src = (b << 32) | a
    out = 0
    for k in range(4):
        sel = (s >> (4 * k)) & 15
        byte = (src >> (8 * (sel & 7))) & 0xFF
        if sel & 8:
            byte = 0xFF if byte & 0x80 else 0
        out |= byte << (8 * k)
    return out


def bam_bytes(nibs):
    """BAM packing: base 2i in the high nibble of byte i, base 2i + 1 in the low."""
    if len(nibs) % 2:
        nibs = list(nibs) + [0]
    return bytes((nibs[2 * i] << 4) | nibs[2 * i + 1] for i in range(len(nibs) // 2))


def decode_chunk(nibs, first, quals, min_qual):
    """The walk's decode of bases first..first+3 of a read (nibbles `nibs`,
    quality bytes `quals`): per base (row, addend, mq-correction flag)."""
    raw = bam_bytes(nibs) + b"\0" * 8
    sb = first >> 1                          # byte of the chunk's first nibble
    sv = int.from_bytes(raw[sb:sb + 4], "little")
    qv = int.from_bytes(bytes(quals[first:first + 4]), "little")
    minq4 = min(max(min_qual, 0), 127) * 0x01010101
    okall = 0xFFFFFFFF if min_qual <= 127 else 0
    comb = COMB_ODD if first & 1 else COMB_EVEN
    code = prmt(prmt(K_LO, K_HI, sv), prmt(K_LO, K_HI, sv >> 8), comb)
    ok = code & (((((qv | 0x80808080) - minq4) & ~qv & 0x80808080) & 0xFFFFFFFF) >> 1) & okall
    qm = qv & (((ok >> 6) * 0x7F) & 0xFFFFFFFF)
    one4 = ok >> 2
    bix = code & 0x03030303
    out = []
    for j in range(4):
        row = prmt(bix, 0, 0x4440 | j)
        add = prmt(qm, one4, j | (12 + j) << 4 | (4 + j) << 8 | (12 + j) << 12)
        out.append((row, add, (ok >> (8 * j + 6)) & 1, prmt(qm, 0, 0x4440 | j)))
    return out


def expected(nib, qbyte, min_qual):
    """PileUp.add: counted when the base is A/C/G/T and the signed quality >= minQual."""
    q = qbyte - 256 if qbyte >= 128 else qbyte
    if NIB[nib] in "ACGT" and q >= min_qual:
        return "ACGT".index(NIB[nib]), q + (1 << 20), 1, q
    return None


@pytest.mark.parametrize("min_qual", [0, 1, 10, 30, 64, 127, 128, 200])
def test_every_code_and_quality_both_parities(min_qual):
    for first in (4, 5):                     # even and odd read offset of the chunk
        for j in range(4):
            for nib in range(16):
                for qbyte in range(256):
                    nibs = [1, 2, 4, 8, 1, 2, 4, 8, 1, 2, 4, 8]
                    quals = [30] * 12
                    nibs[first + j], quals[first + j] = nib, qbyte
                    got = decode_chunk(nibs, first, quals, min_qual)[j]
                    want = expected(nib, qbyte, min_qual)
                    if want is None:
                        assert got[1] == 0 and got[2] == 0 and got[3] == 0, (first, j, NIB[nib], qbyte)
                    else:
                        assert got == want, (first, j, NIB[nib], qbyte, got, want)


def test_random_chunks_match_per_base_rule():
    rng = np.random.Generator(np.random.PCG64(5))
    for _ in range(4000):
        n = 16
        nibs = rng.integers(0, 16, n).tolist()
        quals = rng.integers(0, 256, n).tolist()
        first = int(rng.integers(0, n - 4))
        min_qual = int(rng.integers(0, 130))
        got = decode_chunk(nibs, first, quals, min_qual)
        for j in range(4):
            want = expected(nibs[first + j], quals[first + j], min_qual)
            if want is None:
                assert got[j][1:] == (0, 0, 0)
            else:
                assert got[j] == want


def test_kernel_still_uses_these_formulas():
    """decode_chunk above restates these lines of the walk kernel; a change
    there must be carried over here."""
    src = open(SRC).read()
    for line in ["const uint32_t code = prmt(prmt(kCodeLo, kCodeHi, sv), prmt(kCodeLo, kCodeHi, sv >> 8), comb);",
                 "const uint32_t ok = code & ((((qv | 0x80808080u) - minq4) & ~qv & 0x80808080u) >> 1) & okall;",
                 "const uint32_t qm = qv & ((ok >> 6) * 0x7fu);",
                 "const uint32_t one4 = ok >> 2;",
                 "const uint32_t bix = code & 0x03030303u;",
                 "prmt(qm, one4, (uint32_t)(j | (12 + j) << 4 | (4 + j) << 8 | (12 + j) << 12))",
                 "const uint32_t minq4 = (uint32_t)min(max(P.min_qual, 0), 127) * 0x01010101u;",
                 "const uint32_t okall = P.min_qual <= 127 ? 0xffffffffu : 0u;"]:
        assert line in src, line
