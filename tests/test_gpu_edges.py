"""Edge cases of the pileup path on the GPU against the oracle: an empty read
store, regions without reads, a 1-bp region, unmapped placed reads, every
CIGAR operator (M = X I D N S H P), reads that are all clips, absent
qualities, N bases, flags that validateRead drops (S/BamFile.scala:101-105),
improper pairs, long insertions (string pool), quality bytes of 128 and
above (negative Java bytes), and reads at the contig ends."""
import dataclasses

import numpy as np
import pytest

from pilon_gb300 import _abi
from pilon_gb300.reads import build_store
from tests.helpers import compare_region, oracle_regions

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    from pilon_gb300.engine import Engine
    e = Engine(0)
    yield e
    e.close()


def _ref(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, n)].copy()


class DS:
    def __init__(self, contigs, reads):
        self.contigs, self.reads = contigs, reads


def _records(ref0, ref1):
    rng = np.random.Generator(np.random.PCG64(99))
    s0 = bytes(ref0).decode()
    s1 = bytes(ref1).decode()

    def q(n, lo=20, hi=41):
        return rng.integers(lo, hi, n).tolist()

    recs = []
    # 40x of plain 60M reads over contig 0, so that calls and changes happen
    for p in range(1, 2941, 3):
        seq = list(s0[p - 1:p - 1 + 60])
        if p % 7 == 0:
            seq[30] = "ACGT"[("ACGT".index(seq[30]) + 1) % 4]  # a sequencing error
        if p <= 1600 < p + 60:  # a SNP every read carries
            seq[1600 - p] = "ACGT"[("ACGT".index(s0[1599]) + 2) % 4]
        flag = 0x1 | 0x2 | (0x10 if p % 2 else 0x20)
        recs.append(dict(pos=p, cigar=[(60, "M")], seq="".join(seq), qual=q(60), flag=flag, mapq=60,
                         tlen=(300 if p % 2 == 0 else -300)))
    special = [
        dict(pos=120, cigar=[(20, "="), (1, "X"), (29, "=")], seq=s0[119:139] + "ACGT"[("ACGT".index(s0[139]) + 1) % 4]
             + s0[140:169], qual=q(50)),
        dict(pos=200, cigar=[(20, "M"), (500, "N"), (30, "M")], seq=s0[199:219] + s0[719:749], qual=q(50)),
        dict(pos=260, cigar=[(10, "M"), (2, "P"), (10, "M")], seq=s0[259:279], qual=q(20)),
        dict(pos=300, cigar=[(5, "H"), (40, "M"), (5, "H")], seq=s0[299:339], qual=q(40)),
        dict(pos=350, cigar=[(30, "S")], seq="ACGT" * 7 + "AC", qual=q(30)),                 # all clips
        dict(pos=420, cigar=[(12, "S"), (40, "M"), (9, "S")], seq="T" * 12 + s0[419:459] + "G" * 9, qual=q(61)),
        dict(pos=500, cigar=[], seq="ACGTACGTAC" * 5, qual=q(50), flag=0x4),               # unmapped, placed
        dict(pos=520, cigar=[(50, "M")], seq=s0[519:569], qual=None),                      # absent qualities
        dict(pos=540, cigar=[(50, "M")], seq=s0[539:549] + "NNNNN" + s0[554:589], qual=q(50)),  # N bases
        dict(pos=600, cigar=[(50, "M")], seq=s0[599:649], qual=q(50), mapq=0),
        dict(pos=610, cigar=[(50, "M")], seq=s0[609:659], qual=q(50), flag=0x400),         # duplicate: dropped
        dict(pos=620, cigar=[(50, "M")], seq=s0[619:669], qual=q(50), flag=0x100),         # secondary: dropped
        dict(pos=630, cigar=[(50, "M")], seq=s0[629:679], qual=q(50), flag=0x200),         # QC fail: dropped
        dict(pos=640, cigar=[(50, "M")], seq=s0[639:689], qual=q(50), flag=0x1, tlen=250),  # improper pair
        dict(pos=700, cigar=[(30, "M"), (20, "I"), (30, "M")], seq=s0[699:729] + "ACGTTGCAACGTTGCAACGT"
             + s0[729:759], qual=q(80)),                                                    # long insertion
        dict(pos=760, cigar=[(30, "M"), (15, "D"), (30, "M")], seq=s0[759:789] + s0[804:834], qual=q(60)),
        dict(pos=880, cigar=[(60, "M")], seq=s0[879:939],                                  # negative Java quals
             qual=q(10) + [130, 200, 255, 128, 127, 0, 129, 254] + q(42)),
        dict(pos=900, cigar=[(60, "M")], seq=s0[899:959], qual=[127] * 60),                # the largest accepted
        dict(pos=1, cigar=[(20, "S"), (40, "M")], seq="A" * 20 + s0[0:40], qual=q(60)),    # clip before the start
        dict(pos=2975, cigar=[(26, "M"), (30, "S")], seq=s0[2974:3000] + "C" * 30, qual=q(56)),  # clip past the end
    ]
    recs += special
    recs.sort(key=lambda r: r["pos"])
    for r in recs:
        r["ref_id"] = 0
        r.setdefault("mate_ref_id", 0)
    # one read on contig 1
    recs.append(dict(pos=50, cigar=[(60, "M")], seq=s1[49:109], qual=q(60), ref_id=1, mate_ref_id=1))
    return recs


@pytest.fixture(scope="module")
def edge_ds():
    ref0, ref1 = _ref(3000, 1), _ref(400, 2)
    return DS([ref0, ref1], build_store(_records(ref0, ref1)))


def _regions(ds):
    from pilon_gb300.regions import ReadIndex
    idx = ReadIndex(ds.reads, len(ds.contigs))
    out = []
    for c, s, e in [(0, 1, 3000), (0, 1, 1000), (0, 1001, 2000), (0, 2001, 3000), (0, 1500, 1500),
                    (0, 2900, 3000), (1, 1, 400), (1, 200, 260)]:
        a, b = idx.range_for(c, s, e, ds.contigs[c].size)
        out.append((c, s, e, a, b))
    return out


@pytest.mark.parametrize("batched", [True, False])
def test_edge_cases_match_oracle(engine, edge_ds, batched):
    p = _abi.default_params()
    regions = _regions(edge_ds)
    engine.set_reference(edge_ds.contigs)
    engine.set_reads(edge_ds.reads)
    engine.pileup_regions(regions, p, batched=batched)
    want = oracle_regions(edge_ds, p, regions)
    for r in range(len(regions)):
        compare_region(engine.fetch(r), want[r], f"region {regions[r][:3]}")
    assert want[0].stats.read_count > 900 and want[0].stats.n_changes >= 1


def test_min_qual_and_min_mq_filters(engine, edge_ds):
    p = _abi.default_params(min_qual=25, min_mq=10, flank=3)
    regions = _regions(edge_ds)
    engine.set_reference(edge_ds.contigs)
    engine.set_reads(edge_ds.reads)
    engine.pileup_regions(regions, p)
    want = oracle_regions(edge_ds, p, regions)
    for r in range(len(regions)):
        compare_region(engine.fetch(r), want[r], f"region {regions[r][:3]}")


def test_empty_read_store(engine, edge_ds):
    empty = edge_ds.reads.subset(np.arange(0))
    ds = DS(edge_ds.contigs, empty)
    regions = [(0, 1, 3000, 0, 0), (1, 1, 400, 0, 0)]
    p = _abi.default_params()
    engine.set_reference(ds.contigs)
    engine.set_reads(empty)
    engine.pileup_regions(regions, p)
    want = oracle_regions(ds, p, regions)
    for r in range(len(regions)):
        got = engine.fetch(r)
        compare_region(got, want[r], f"empty store region {r}")
        assert got.stats.read_count == 0


def _run_tuned(engine, ds, p, variant, label):
    regions = _regions(ds)
    engine.set_reference(ds.contigs)
    engine.set_reads(ds.reads)
    engine.set_tuning(1024, 16, variant)
    try:
        engine.pileup_regions(regions, p)
        want = oracle_regions(ds, p, regions)
        for r in range(len(regions)):
            compare_region(engine.fetch(r), want[r], f"{label} variant {variant} region {regions[r][:3]}")
    finally:
        engine.set_tuning(2048, 16, 0)


@pytest.mark.parametrize("variant", [0, 2])
@pytest.mark.parametrize("min_qual", [0, 1, 127, 128, 200])
def test_min_qual_bounds(engine, edge_ds, min_qual, variant):
    """minQual at the bounds of a signed quality byte: 127 still accepts
    quality 127, 128 and above accept nothing; quality bytes of 128 and above
    are rejected at every minQual."""
    _run_tuned(engine, edge_ds, _abi.default_params(min_qual=min_qual), variant, f"minQual {min_qual}")


@pytest.mark.parametrize("variant", [0, 2])
@pytest.mark.parametrize("mapq", [0, 17, 255])
def test_store_wide_mapq(engine, edge_ds, mapq, variant):
    """The walk adds the reads of the store's most common adjusted mapq with
    one atomic per base and corrects the others' sums by their difference to
    it; every most common mapq, 0 and 255 included, gives the oracle's sums.
    A few reads keep mapq 60 beside the others."""
    mq = np.full(edge_ds.reads.n_reads, mapq, np.uint8)
    mq[::11] = 60
    ds = DS(edge_ds.contigs, dataclasses.replace(edge_ds.reads, mapq=mq))
    _run_tuned(engine, ds, _abi.default_params(), variant, f"mapq {mapq}")
