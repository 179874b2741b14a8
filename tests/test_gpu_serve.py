"""Serving: requests batched together (continuous batching over two engine
contexts) must get exactly the answers they get alone."""
import pytest

from pilon_gb300 import synth
from pilon_gb300.serve import Request, Server, poisson_requests

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix():
    ds = synth.generate(3, scale=0.02)
    lens = [c.size for c in ds.contigs]
    sched = poisson_requests(lens, rate=2000.0, duration=0.03, seed=7, min_len=2_000, max_len=60_000)
    assert len(sched) >= 20
    mix = Server(ds.names, ds.contigs, ds.reads, n_workers=2, budget_positions=300_000)
    try:
        futs = [mix.submit(Request(r.contig, r.start, r.stop, rid=r.rid)) for _, r in sched]
        got = [f.exception() or f.result() for f in futs]
        assert mix.batches < len(sched)  # requests really were batched
    finally:
        mix.close()
    alone = Server(ds.names, ds.contigs, ds.reads, n_workers=1, budget_positions=1, batched=False)
    try:
        ref = []
        for _, r in sched:
            f = alone.submit(Request(r.contig, r.start, r.stop, rid=r.rid))
            ref.append(f.exception() or f.result())
    finally:
        alone.close()
    n_ok = 0
    for a, b in zip(got, ref):
        if isinstance(a, Exception) or isinstance(b, Exception):
            # a target the reference would crash on fails alone and in the mix
            assert isinstance(a, IndexError) and isinstance(b, IndexError)
            continue
        assert a.fasta == b.fasta and a.changes == b.changes and a.vcf == b.vcf, a.rid
        n_ok += 1
    assert n_ok >= len(sched) // 2 and sum(len(a.vcf) for a in got if not isinstance(a, Exception)) > 0
