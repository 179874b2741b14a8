"""K-mer tally and break detection on the GPU path against the oracle."""
import numpy as np
import pytest

from oracle import oracle
from pilon_gb300 import _abi, synth
from tests.breaks_host import possible_breaks, region_arrays
from pilon_gb300.regions import ReadIndex, plan_regions

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    from pilon_gb300.engine import Engine
    e = Engine(0)
    yield e
    e.close()


@pytest.fixture(scope="module")
def euk():
    # the eukaryotic workload scaled to 600 kb: repeats with mapq 0-3, 10-200 bp indels
    return synth.generate(4, scale=0.005)


def edge_set(edges):
    return {(int(e["window"]), int(e["key_hi"]), int(e["key_lo"]), int(e["next"]), int(e["alt"]), int(e["depth"]),
             int(e["weight"])) for e in edges}


def test_breaks_match_oracle(engine, euk):
    ds = euk
    p = _abi.default_params()
    regions = plan_regions(ds.reads, [c.size for c in ds.contigs], chunk_size=200_000)
    engine.set_reference(ds.contigs)
    engine.set_reads(ds.reads)
    engine.pileup_regions(regions, p)
    total = 0
    for r, (c, s, e, a, b) in enumerate(regions):
        x = engine.fetch(r)
        cov, bad, clips, frag = region_arrays(x.count, x.deletions, x.bad_pair, x.clips, x.call, x.indel_len,
                                              x.stats.read_count)
        got = possible_breaks(cov, bad, clips, frag, ds.contigs[c][s - 1:e], s, e)
        want = oracle.region_breaks(ds.reads, p, ds.contigs[c], c, s, e, a, b)
        assert got == want, (r, got[:5], want[:5])
        total += len(want)
    assert total > 0


def test_kmer_tally_matches_oracle(engine, euk):
    ds = euk
    p = _abi.default_params()
    idx = ReadIndex(ds.reads, len(ds.contigs))
    n = ds.contigs[0].size
    # windows around planted-indel neighbourhoods: reads overlapping [x - 500, x + 500]
    wins = []
    for (pos, kind, ref, alt) in ds.variants[0][:40]:
        a, b = idx.range_for(0, max(1, pos - 500), min(n, pos + 500), n, slop=0)
        wins.append((a, b))
    engine.set_reference(ds.contigs)
    engine.set_reads(ds.reads)
    for K in (31, 19):
        got = engine.kmer_tally(wins, K, p)
        want = oracle.kmer_tally(ds.reads, p, wins, K)
        assert len(got) > 1000
        assert edge_set(got) == edge_set(want)


def test_kmer_tally_exotic_kmers(engine, cfg1):
    # reads with N bases give K-mers that cannot be 2-bit packed
    ds = cfg1
    r = ds.reads
    seq = r.seq.copy()
    rng = np.random.Generator(np.random.PCG64(5))
    hit = rng.choice(r.n_reads, size=r.n_reads // 5, replace=False)
    for i in hit[:2000].tolist():  # put an N (code 15) at base 40 of 2,000 reads
        o = int(r.seq_off[i]) + 20
        seq[o] = (seq[o] & 0x0F) | 0xF0
    r2 = r.subset(np.arange(r.n_reads))
    r2.seq = seq
    engine.set_reference(ds.contigs)
    engine.set_reads(r2)
    p = _abi.default_params()
    wins = [(0, 3000), (3000, 6000), (5000, 9000)]
    got = engine.kmer_tally(wins, 25, p, min_depth=2)
    want = oracle.kmer_tally(r2, p, wins, 25, min_depth=2)
    assert edge_set(got) == edge_set(want)
    assert any((int(e["key_hi"]) >> 60) == 15 or "F" in format(int(e["key_hi"]), "016x") for e in want)


def test_assembler_graph(engine, cfg1):
    from tests.assembler_host import Assembler
    engine.set_reference(cfg1.contigs)
    engine.set_reads(cfg1.reads)
    asm = Assembler(engine, K=21)
    w = asm.add_reads(100, 900)
    kg, ag = asm.build_graph(_abi.default_params())[w]
    assert len(kg) > 100
    for k, nxt in list(kg.items())[:50]:
        assert nxt[:-1] == k[1:] and len(nxt) == 21


def _device_breaks_vs_oracle(engine, ds, regions, p):
    engine.set_reference(ds.contigs)
    engine.set_reads(ds.reads)
    engine.pileup_regions(regions, p)
    got = engine.find_breaks(p.min_min_depth)
    total = 0
    for r, (c, s, e, a, b) in enumerate(regions):
        try:
            want = oracle.region_breaks(ds.reads, p, ds.contigs[c], c, s, e, a, b)
        except IndexError:  # the reference throws on this region: no breaks from the device either
            want = []
        assert got.get(r, []) == want, (r, got.get(r, [])[:5], want[:5])
        total += len(want)
    return total


def test_device_breaks_match_oracle(engine, euk):
    """pg_find_breaks (GenomeRegion.possibleBreaks on the device) on the
    eukaryotic workload, with runs of N written into the reference so that the
    gap rules (>= 10 bases, breaks within 300 bases of a gap dropped) apply."""
    ds = euk
    refs = [c.copy() for c in ds.contigs]
    n = refs[0].size
    rng = np.random.Generator(np.random.PCG64(11))
    for x in rng.choice(np.arange(1000, n - 1000), size=12, replace=False).tolist():
        refs[0][x:x + int(rng.integers(5, 60))] = ord("N")
    from types import SimpleNamespace
    ds2 = SimpleNamespace(contigs=refs, reads=ds.reads)
    p = _abi.default_params()
    regions = plan_regions(ds.reads, [c.size for c in refs], chunk_size=200_000)
    assert _device_breaks_vs_oracle(engine, ds2, regions, p) > 0


def test_device_breaks_many_contigs(engine):
    ds = synth.generate(3, scale=0.02)
    p = _abi.default_params()
    regions = plan_regions(ds.reads, [c.size for c in ds.contigs])
    _device_breaks_vs_oracle(engine, ds, regions, p)
    p2 = _abi.default_params(min_min_depth=12)
    _device_breaks_vs_oracle(engine, ds, regions, p2)


def test_kmer_tally_over_device_break_windows(engine, euk):
    """pg_kmer_tally_breaks builds one window per device break candidate and
    tallies it; the windows equal the host index's read ranges, so the edges
    equal pg_kmer_tally over the host windows and the oracle's."""
    ds = euk
    p = _abi.default_params()
    lens = [c.size for c in ds.contigs]
    regions = plan_regions(ds.reads, lens, chunk_size=200_000)
    engine.set_reference(ds.contigs)
    engine.set_reads(ds.reads)
    engine.pileup_regions(regions, p)
    brk = engine.find_breaks(p.min_min_depth)
    idx = ReadIndex(ds.reads, len(ds.contigs))
    wins = []
    for r in sorted(brk):
        c = regions[r][0]
        for (s, e) in brk[r]:
            wins.append(idx.range_for(c, s, e, lens[c], slop=500))
    assert len(wins) > 10
    nw, got = engine.kmer_tally_breaks(31, p, radius=500)
    assert nw == len(wins)
    want = engine.kmer_tally(wins, 31, p)
    assert edge_set(got) == edge_set(want)
    assert edge_set(oracle.kmer_tally(ds.reads, p, wins[:8], 31)) == edge_set(
        [e for e in got if int(e["window"]) < 8])


def wide_edge_set(edges):
    return {(int(e["window"]), int(e["key0"]), int(e["key1"]), int(e["key2"]), int(e["key3"]), int(e["next"]),
             int(e["alt"]), int(e["depth"]), int(e["weight"])) for e in edges}


def test_kmer_tally_wide_matches_oracle(engine, euk):
    """pg_kmer_tally_wide at Pilon's default K = 47 (S/Assembler.scala:25), at
    K = 63 and at K = 32 (the first K a 64-bit key cannot hold) equals the
    oracle's tally; at K = 31 it equals pg_kmer_tally's edges."""
    ds = euk
    p = _abi.default_params()
    idx = ReadIndex(ds.reads, len(ds.contigs))
    n = ds.contigs[0].size
    wins = [idx.range_for(0, max(1, pos - 500), min(n, pos + 500), n, slop=0)
            for (pos, kind, ref, alt) in ds.variants[0][:30]]
    engine.set_reference(ds.contigs)
    engine.set_reads(ds.reads)
    for K in (47, 63, 32):
        got = engine.kmer_tally(wins, K, p)
        want = oracle.kmer_tally_wide(ds.reads, p, wins, K)
        assert len(got) > 1000, K
        assert wide_edge_set(got) == wide_edge_set(want), K
    narrow = engine.kmer_tally(wins, 31, p)
    wide = engine.kmer_tally(wins, 31, p, wide=True)
    assert {(w, a, b, x, y, d, g) for (w, a, b, c2, d2, x, y, d, g) in wide_edge_set(wide)} == edge_set(narrow)
    assert all(int(e["key2"]) == 0 and int(e["key3"]) == 0 for e in wide)


def test_kmer_tally_wide_exotic_kmers(engine, cfg1):
    """K = 47 with reads holding N bases: the K-mers with N are tallied in the
    4-word exotic tables."""
    ds = cfg1
    r = ds.reads
    seq = r.seq.copy()
    rng = np.random.Generator(np.random.PCG64(5))
    hit = rng.choice(r.n_reads, size=r.n_reads // 5, replace=False)
    for i in hit[:2000].tolist():
        o = int(r.seq_off[i]) + 20
        seq[o] = (seq[o] & 0x0F) | 0xF0
    r2 = r.subset(np.arange(r.n_reads))
    r2.seq = seq
    engine.set_reference(ds.contigs)
    engine.set_reads(r2)
    p = _abi.default_params()
    wins = [(0, 3000), (3000, 6000), (5000, 9000)]
    got = engine.kmer_tally(wins, 47, p, min_depth=2)
    want = oracle.kmer_tally_wide(r2, p, wins, 47, min_depth=2)
    assert wide_edge_set(got) == wide_edge_set(want)
    assert any("f" in "".join(format(int(e[f"key{q}"]), "016x") for q in range(3)) for e in want)


def test_kmer_tally_full_tables_counted_again(engine, cfg1):
    """Windows whose reads share no K-mers fill tables sized at a quarter of
    their K-mer events: they write no edges in the first pass and are counted
    again in larger tables after the other windows, and every window's edges
    equal the oracle's."""
    ds = cfg1
    r = ds.reads
    assert np.all(np.diff(r.seq_off[:1501]) > 0)
    seq = r.seq.copy()
    rng = np.random.Generator(np.random.PCG64(11))
    codes = np.array([1, 2, 4, 8], np.uint8)
    lo, hi = int(r.seq_off[0]), int(r.seq_off[1500])
    seq[lo:hi] = (codes[rng.integers(0, 4, hi - lo)] << 4) | codes[rng.integers(0, 4, hi - lo)]
    r2 = r.subset(np.arange(r.n_reads))
    r2.seq = seq
    engine.set_reference(ds.contigs)
    engine.set_reads(r2)
    p = _abi.default_params()
    wins = [(0, 1500), (1500, 3000), (100, 1400)]
    got = engine.kmer_tally(wins, 25, p, min_depth=1)
    want = oracle.kmer_tally(r2, p, wins, 25, min_depth=1)
    assert edge_set(got) == edge_set(want)
    _, _, distinct, _, batches = engine.last_tally_stats()
    assert batches >= 2  # the first pass, then the full windows again
    assert distinct > 300_000
