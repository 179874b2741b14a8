"""pg_region_fixes and pg_changes_lines (host C++, no device) against a
Python restatement of GenomeRegion's fix lists, fixFixList, fixIssues and the
changes lines (S/GenomeRegion.scala:307-380, 557-621, 645-657) on random
change lists: SNP, AMB (as a base or an IUPAC code), insertions, deletions
that run past the region or the contig, excluded loci, empty lists."""
import numpy as np
import pytest

from pilon_gb300 import _abi
from pilon_gb300.engine import changes_lines, region_fixes
from pilon_gb300.polish import Fix, fix_fix_list

ACGT = "ACGT"
IUPAC = {1: "A", 2: "C", 4: "G", 8: "T", 5: "R", 10: "Y", 6: "S", 9: "W", 12: "K", 3: "M", 14: "B", 13: "D",
         11: "H", 7: "V", 15: "N"}  # Bases.toIUPAC (S/Bases.scala:85-88)


def _fix_issues(bases, start, fixes):
    """fixIssues step by step: fixFixList, then from the last fix to the first."""
    nb = bytearray(bases)
    for f in reversed(fix_fix_list(fixes)):
        s = f.locus - start
        if len(f.was) == len(f.patch):
            nb[s:s + len(f.patch)] = f.patch.encode()
        else:
            nb = nb[:s] + f.patch.encode() + nb[s + len(f.was):]
    return bytes(nb)


def _lists(changes, chars, contig, start, fix_snps, fix_indels, iupac, long_read, excluded):
    """identifyAndFixIssues' snp and small lists, each last change first."""
    snp, small = [], []
    for ch in changes:
        loc, f, ilen, ioff = int(ch["locus"]), int(ch["call"]), int(ch["indel_len"]), int(ch["ins_str"])
        if excluded is not None and excluded[loc - start]:
            continue
        k = (f >> 9) & 7
        rb = chr(contig[loc - 1]).upper()
        cb = ACGT[f & 3] if f & _abi.PG_CALL_HAS_BASE else "N"
        if k == _abi.PG_CHANGE_SNP and fix_snps:
            snp.append(Fix(loc, rb, cb))
        elif k == _abi.PG_CHANGE_AMB and fix_snps and not long_read:
            if iupac:
                small.append(Fix(loc, rb, IUPAC[(1 << (f & 3)) | (1 << ((f >> 2) & 3))]))
            else:
                snp.append(Fix(loc, rb, cb))
        elif k == _abi.PG_CHANGE_INS and fix_indels:
            small.append(Fix(loc, "", chars[ioff:ioff + ilen].decode()))
        elif k == _abi.PG_CHANGE_DEL and fix_indels:
            small.append(Fix(loc, bytes(contig[loc - 1:loc - 1 + ilen]).decode(), ""))
    return snp[::-1], small[::-1]


def _lines(fixes, name, new_name, offset):
    out, delta = [], 0
    for f in fix_fix_list(fixes):
        lw, lp = len(f.was), len(f.patch)
        nl = f.locus + delta + offset
        out.append(f"{name}:{f.locus}{'' if lw < 2 else f'-{f.locus + lw - 1}'} "
                   f"{new_name}:{nl}{'' if lp < 2 else f'-{nl + lp - 1}'} {f.was or '.'} {f.patch or '.'}\n")
        delta += lp - lw
    return "".join(out).encode()


def _decode(fixes, text):
    return [(int(f["list"]), Fix(int(f["locus"]), text[f["was_off"]:f["was_off"] + f["was_len"]].decode(),
                                 text[f["patch_off"]:f["patch_off"] + f["patch_len"]].decode())) for f in fixes]


def _random_case(rng):
    contig = rng.choice(np.frombuffer(b"ACGTacgtN", np.uint8), int(rng.integers(30, 400)))
    n = contig.size
    start = int(rng.integers(1, n // 2))
    stop = int(rng.integers(start, n + 1))
    loci = np.sort(rng.choice(np.arange(start, stop + 1), min(stop - start + 1, int(rng.integers(0, 25))),
                              replace=False))
    ch = np.zeros(loci.size, _abi.change_dtype())
    pool = bytearray()
    for k, loc in enumerate(loci):
        kind = int(rng.choice([_abi.PG_CHANGE_SNP, _abi.PG_CHANGE_AMB, _abi.PG_CHANGE_INS, _abi.PG_CHANGE_DEL]))
        b, alt = int(rng.integers(0, 4)), int(rng.integers(0, 4))
        has = _abi.PG_CALL_HAS_BASE if (kind != _abi.PG_CHANGE_SNP or rng.random() < 0.9) else 0
        call = (kind << 9) | b | (alt << 2) | has
        ilen, ioff = 0, -1
        if kind == _abi.PG_CHANGE_INS:
            ilen, ioff = int(rng.integers(1, 8)), len(pool)
            pool += bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), ilen))
        elif kind == _abi.PG_CHANGE_DEL:
            ilen = int(rng.integers(1, 30))  # may run past the region and the contig
        ch[k] = (0, loc, call, ilen, ioff, 0)
    return contig, start, stop, ch, bytes(pool)


def test_region_fixes_and_changes_lines_match_restatement():
    rng = np.random.default_rng(5)
    for trial in range(600):
        contig, start, stop, ch, pool = _random_case(rng)
        opts = dict(fix_snps=bool(rng.random() < 0.8), fix_indels=bool(rng.random() < 0.8),
                    iupac=bool(rng.random() < 0.3), long_read=bool(rng.random() < 0.2))
        excluded = (rng.random(stop - start + 1) < 0.1) if rng.random() < 0.3 else None
        fixes, text, bases_snp, bases = region_fixes(ch, pool, contig, start, stop, excluded=excluded, **opts)
        snp, small = _lists(ch, pool, contig, start, excluded=excluded, **opts)
        got = _decode(fixes, text)
        assert got == [(0, f) for f in snp] + [(1, f) for f in small], trial
        orig = bytes(contig[start - 1:stop])
        want_snp = _fix_issues(orig, start, snp)
        assert bases_snp == want_snp, trial
        assert bases == _fix_issues(want_snp, start, small), trial
        offset = int(rng.integers(-50, 50))
        assert changes_lines(fixes, text, "ctg", "ctg_pilon", offset) == \
            _lines(snp + small, "ctg", "ctg_pilon", offset), trial


def test_changes_lines_resolve_overlaps_with_big_fixes():
    """fixFixList over snp ++ small ++ big: of two overlapping fixes the one
    with more bases stays, the first on a tie (S/GenomeRegion.scala:557-593)."""
    rng = np.random.default_rng(9)
    for trial in range(300):
        fixes = []
        for _ in range(int(rng.integers(0, 12))):
            loc = int(rng.integers(1, 60))
            was = "".join(rng.choice(list("ACGT"), int(rng.integers(0, 6))))
            patch = "".join(rng.choice(list("ACGTN"), int(rng.integers(0, 6))))
            fixes.append((int(rng.integers(0, 3)), Fix(loc, was, patch)))
        arr = np.zeros(len(fixes), _abi.fix_dtype())
        text = bytearray()
        for k, (lst, f) in enumerate(fixes):
            arr[k] = (f.locus, lst, len(text), len(f.was), len(text) + len(f.was), len(f.patch))
            text += (f.was + f.patch).encode()
        assert changes_lines(arr, bytes(text), "c", "c_pilon", 3) == _lines([f for _, f in fixes], "c", "c_pilon", 3)


def test_region_fixes_refuse_changes_outside_the_region():
    from pilon_gb300.engine import EngineError
    contig = np.frombuffer(b"ACGTACGTAC", np.uint8)
    ch = np.zeros(1, _abi.change_dtype())
    ch[0] = (0, 9, (_abi.PG_CHANGE_SNP << 9) | _abi.PG_CALL_HAS_BASE, 0, -1, 0)
    with pytest.raises(EngineError):
        region_fixes(ch, b"", contig, 2, 8)
    ch[0] = (0, 5, (_abi.PG_CHANGE_INS << 9) | _abi.PG_CALL_HAS_BASE, 4, 0, 0)  # insertion past its pool
    with pytest.raises(EngineError):
        region_fixes(ch, b"AC", contig, 2, 8)
    empty = region_fixes(np.zeros(0, _abi.change_dtype()), b"", contig, 2, 8)
    assert empty[0].size == 0 and empty[2] == empty[3] == b"CGTACGT"
