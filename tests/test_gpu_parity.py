"""GPU engine vs the CPU oracle, through the C ABI: every pileup field, call
flag, score, indel string and region statistic must be bit-identical."""
import numpy as np
import pytest

from pilon_gb300 import _abi, synth
from tests.helpers import compare_region, oracle_regions, plan

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    from pilon_gb300.engine import Engine
    e = Engine(0)
    yield e
    e.close()


def run_both(engine, ds, params, regions, batched=True):
    engine.set_reference(ds.contigs)
    engine.set_reads(ds.reads)
    engine.pileup_regions(regions, params, batched=batched)
    ora = oracle_regions(ds, params, regions)
    for r in range(len(regions)):
        compare_region(engine.fetch(r), ora[r], label=f"region {r}")
    return ora


def test_cfg1_single_region(engine, cfg1):
    p = _abi.default_params()
    ora = run_both(engine, cfg1, p, plan(cfg1))
    assert ora[0].stats.n_changes >= 20


def test_cfg1_chunked_regions_plain_and_batched(engine, cfg1):
    p = _abi.default_params()
    regions = plan(cfg1, chunk_size=7000)
    assert len(regions) > 5
    run_both(engine, cfg1, p, regions, batched=True)
    run_both(engine, cfg1, p, regions, batched=False)


@pytest.mark.parametrize("opts", [dict(min_mq=20), dict(min_qual=25), dict(flank=0), dict(flank=40),
                                  dict(nonpf=1, duplicates=1), dict(old_indel=1), dict(fix_amb=1),
                                  dict(min_depth=12.0), dict(default_qual=30)])
def test_cfg1_options(engine, cfg1, opts):
    run_both(engine, cfg1, _abi.default_params(**opts), plan(cfg1))


def test_cfg2_scaled(engine):
    ds = synth.generate(2, scale=0.02)  # 100 kb at 100x, mapq-0 reads, indel errors
    run_both(engine, ds, _abi.default_params(), plan(ds, chunk_size=30_000))


def test_cfg3_many_contigs(engine):
    ds = synth.generate(3, scale=0.01)  # 30 contigs, 1% variants
    regions = plan(ds)
    run_both(engine, ds, _abi.default_params(), regions, batched=True)
    run_both(engine, ds, _abi.default_params(), regions, batched=False)


def test_long_read_modes(engine, cfg1):
    for lr in (_abi.PG_NANOPORE, _abi.PG_PACBIO):
        p = _abi.default_params(long_read=lr, bam_type=_abi.PG_BAM_UNPAIRED)
        run_both(engine, cfg1, p, plan(cfg1, chunk_size=20_000))


@pytest.mark.parametrize("tile,warps,variant", [(1024, 8, 0), (1024, 16, 1), (2048, 8, 2), (4096, 16, 0),
                                                (512, 16, 1), (4096, 8, 2), (256, 4, 1), (2048, 16, 2),
                                                (256, 8, 2), (512, 8, 2), (1024, 8, 3), (2048, 16, 3),
                                                (256, 16, 3), (4096, 16, 3), (512, 4, 0), (2048, 8, 1)])
def test_walk_tunings_bit_exact(engine, cfg1, tile, warps, variant):
    engine.set_tuning(tile, warps, variant)
    try:
        run_both(engine, cfg1, _abi.default_params(), plan(cfg1, chunk_size=12_000))
    finally:
        engine.set_tuning(2048, 16, 0)


@pytest.mark.parametrize("variant", [0, 2])
def test_high_coverage_multi_pass(engine, variant):
    # 2,000x on a short contig: a 4,096-position tile sees ~55k reads per pass limit region
    w = synth.workload(1, scale=0.04)
    w.coverage = 2000.0
    ds = synth.generate(w)
    engine.set_tuning(2048, 16, variant)
    try:
        run_both(engine, ds, _abi.default_params(), plan(ds))
    finally:
        engine.set_tuning(2048, 16, 0)


@pytest.mark.parametrize("variant", [2, 3])
def test_cfg2_scaled_variants(engine, variant):
    # mapq-0 reads and clipped reads beside the mapq-60 majority
    ds = synth.generate(2, scale=0.02)
    engine.set_tuning(1024, 16, variant)
    try:
        run_both(engine, ds, _abi.default_params(), plan(ds, chunk_size=30_000))
        run_both(engine, ds, _abi.default_params(min_qual=30, min_mq=1), plan(ds, chunk_size=30_000))
    finally:
        engine.set_tuning(2048, 16, 0)


def test_graph_replay_bit_exact(engine, cfg1):
    """The batched path records a CUDA graph on the second identical call and
    replays it afterwards; every replay must give the same results, also after
    a different plan ran in between."""
    p = _abi.default_params()
    a = plan(cfg1, chunk_size=9000)
    b = plan(cfg1, chunk_size=13000)
    engine.set_reference(cfg1.contigs)
    engine.set_reads(cfg1.reads)
    ora = oracle_regions(cfg1, p, a)
    for k in range(4):
        engine.pileup_regions(a, p, batched=True)
        for r in range(len(a)):
            compare_region(engine.fetch(r), ora[r], label=f"call {k} region {r}")
    engine.pileup_regions(b, p, batched=True)
    engine.pileup_regions(a, p, batched=True)
    for r in range(len(a)):
        compare_region(engine.fetch(r), ora[r], label=f"after switch region {r}")


def test_fetch_all_equals_per_region(engine, cfg1):
    """pg_fetch_all returns every region's arrays, one region after another."""
    from pilon_gb300.engine import RegionArrays
    regions = plan(cfg1, chunk_size=12_000)
    engine.set_reference(cfg1.contigs)
    engine.set_reads(cfg1.reads)
    engine.pileup_regions(regions, _abi.default_params())
    total = sum(e - s + 1 for (c, s, e, a, b) in regions)
    allr = engine.fetch_all(RegionArrays(total))
    off = 0
    for r, (c, s, e, a, b) in enumerate(regions):
        one = engine.fetch(r)
        n = e - s + 1
        for f in ("count", "qual_sum"):
            assert np.array_equal(getattr(allr, f)[4 * off:4 * (off + n)], getattr(one, f)), (r, f)
        for f in list(RegionArrays.I32) + ["call", "score"]:
            assert np.array_equal(getattr(allr, f)[off:off + n], getattr(one, f)), (r, f)
        off += n


def test_graph_not_replayed_after_reallocation(cfg1):
    """A recorded graph holds the addresses of the context's buffers.  A call
    that grows one of them (here a plan with four times the regions, on the
    per-region path) must end the replays: the next batched call of the first
    plan runs its launches again and matches the oracle, and replays resume
    only after the plan has been recorded anew (a call marks a plan, the next
    identical one records it, later ones replay it)."""
    from pilon_gb300.engine import Engine
    p = _abi.default_params()
    a = plan(cfg1, chunk_size=9000)
    b = plan(cfg1, chunk_size=2000)
    assert len(b) >= 4 * len(a)
    ora_a = oracle_regions(cfg1, p, a)
    ora_b = oracle_regions(cfg1, p, b)
    eng = Engine(0)
    try:
        eng.set_reference(cfg1.contigs)
        eng.set_reads(cfg1.reads)

        def check(regs, ora, label):
            for r in range(len(regs)):
                compare_region(eng.fetch(r), ora[r], label=f"{label} region {r}")
        for k in range(6):  # marked, recorded, replayed (later when a first call grows its buffers)
            eng.pileup_regions(a, p, batched=True)
            check(a, ora_a, f"a{k}")
            if eng.graph_replays():
                break
        r0 = eng.graph_replays()
        assert r0 >= 1
        eng.pileup_regions(b, p, batched=False)
        check(b, ora_b, "b plain")
        eng.pileup_regions(a, p, batched=True)
        check(a, ora_a, "a after b")
        assert eng.graph_replays() == r0, "a graph with freed buffers was replayed"
        eng.pileup_regions(b, p, batched=True)
        check(b, ora_b, "b batched")
        for k in range(4):  # marked, recorded, replayed
            eng.pileup_regions(a, p, batched=True)
            check(a, ora_a, f"a again {k}")
        assert eng.graph_replays() > r0
    finally:
        eng.close()


def test_region_range_of_another_reference_refused(cfg1):
    """A region whose read range holds reads of another reference is refused
    (PG_ERR_ARG), in a store with one run per reference and in a store whose
    references interleave; a well-formed call afterwards still matches the
    oracle."""
    from pilon_gb300.engine import Engine, EngineError
    from pilon_gb300.reads import concat_stores
    p = _abi.default_params()
    one = cfg1.reads
    two = concat_stores([one, one])
    two.ref_id[one.n_reads:] = 1
    two.mate_ref_id[one.n_reads:] = 1
    n = one.n_reads
    size = cfg1.contigs[0].size
    eng = Engine(0)
    try:
        eng.set_reference([cfg1.contigs[0], cfg1.contigs[0]])
        eng.set_reads(two)
        for bad in ([(0, 1, size, 0, n + 10)], [(1, 1, size, n - 5, 2 * n)], [(1, 1, size, 0, n)]):
            with pytest.raises(EngineError) as ei:
                eng.pileup_regions(bad, p, batched=True)
            assert ei.value.status == _abi.PG_ERR_ARG and "another reference" in str(ei.value)
        good = [(0, 1, size, 0, n), (1, 1, size, n, 2 * n)]
        eng.pileup_regions(good, p, batched=True)
        ora = oracle_regions(cfg1, p, [(0, 1, size, 0, n)])
        compare_region(eng.fetch(0), ora[0], label="contig 0")
        compare_region(eng.fetch(1), ora[0], label="contig 1")
        # references interleaved (1 before 0): every read of a range is checked
        swapped = concat_stores([one, one])
        swapped.ref_id[:n] = 1
        swapped.mate_ref_id[:n] = 1
        eng.set_reads(swapped)
        with pytest.raises(EngineError) as ei:
            eng.pileup_regions([(0, 1, size, n - 3, 2 * n)], p, batched=True)
        assert ei.value.status == _abi.PG_ERR_ARG
        eng.pileup_regions([(1, 1, size, 0, n), (0, 1, size, n, 2 * n)], p, batched=True)
        compare_region(eng.fetch(1), ora[0], label="swapped contig 0")
    finally:
        eng.close()


def test_fetch_changes_equals_call_arrays(engine):
    """pg_fetch_changes returns exactly the positions whose call carries a
    change, in region and locus order, with the calls, indel lengths and
    insertion strings of the per-region arrays."""
    ds = synth.generate(3, scale=0.01)
    regions = plan(ds)
    engine.set_reference(ds.contigs)
    engine.set_reads(ds.reads)
    engine.pileup_regions(regions, _abi.default_params())
    changes, chars = engine.fetch_changes()
    want = []
    for r, (c, s, e, a, b) in enumerate(regions):
        x = engine.fetch(r)
        for i in np.nonzero((x.call >> 9) & 7)[0].tolist():
            want.append((r, s + i, int(x.call[i]), int(x.indel_len[i]), x.insertion(i)))
    got = [(int(ch["region"]), int(ch["locus"]), int(ch["call"]), int(ch["indel_len"]),
            chars[int(ch["ins_str"]):int(ch["ins_str"]) + int(ch["indel_len"])].decode() if ch["ins_str"] >= 0 else "")
           for ch in changes]
    assert len(want) > 100 and got == want


def test_packed_upload(engine, cfg1):
    """pg_set_reads_packed derives the offsets and alignment ends of a packed
    store on the device: the same pileups as the full upload, also when the
    derived fields are left out, and a store whose lengths do not fill its
    arrays is refused."""
    import copy
    from pilon_gb300.engine import EngineError
    p = _abi.default_params()
    regions = plan(cfg1, chunk_size=12_000)
    ora = oracle_regions(cfg1, p, regions)
    engine.set_reference(cfg1.contigs)
    lean = copy.copy(cfg1.reads)
    for f in ("aend", "cigar_off", "seq_off", "qual_off"):
        setattr(lean, f, np.zeros(0, getattr(cfg1.reads, f).dtype))
    for store in (cfg1.reads, lean):
        engine.set_reads(store, packed=True)
        engine.pileup_regions(regions, p, batched=True)
        for r in range(len(regions)):
            compare_region(engine.fetch(r), ora[r], label=f"packed region {r}")
    gappy = copy.copy(cfg1.reads)
    gappy.qual = np.concatenate([cfg1.reads.qual, np.zeros(7, np.uint8)])
    with pytest.raises(EngineError):
        engine.set_reads(gappy, packed=True)
    engine.set_reads(cfg1.reads)
