"""Serving through the C ABI (pg_serve_*): every answer must equal the
oracle's `pilon --targets` run of that target, and requests batched together
(continuous batching over two engine contexts, admitted by device bytes) must
get exactly the answers they get alone on the plain path."""
import numpy as np
import pytest

from oracle import oracle
from pilon_gb300 import _abi, synth
from pilon_gb300.regions import ReadIndex
from pilon_gb300.serve import Request, Server, poisson_requests

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def draft():
    return synth.generate(3, scale=0.02)


def _variant_records(vcf):
    """The records a served delta keeps: ALT not "." (and no <DUP> records)."""
    out = []
    for line in vcf.split(b"\n"):
        if line:
            f = line.split(b"\t")
            if f[4] != b"." and f[4] != b"<DUP>":
                out.append(line + b"\n")
    return b"".join(out)


def _serve(ds, sched, **kw):
    srv = Server(ds.names, ds.contigs, ds.reads, **kw)
    try:
        futs = [srv.submit(Request(r.contig, r.start, r.stop, rid=r.rid)) for _, r in sched]
        got = [f.exception() or f.result() for f in futs]
        return got, srv.batches, srv.peak_in_flight_bytes()
    finally:
        srv.close()


def test_answers_equal_target_runs_and_same_alone_and_in_the_mix(draft):
    ds = draft
    lens = [c.size for c in ds.contigs]
    sched = poisson_requests(lens, rate=2000.0, duration=0.03, seed=7, min_len=2_000, max_len=60_000)
    assert len(sched) >= 20
    budget = 12_000_000  # bytes: a few requests per batch
    mix, batches, peak = _serve(ds, sched, n_workers=2, budget_bytes=budget)
    assert batches < len(sched)  # requests really were batched
    assert 0 < peak <= budget
    alone, _, _ = _serve(ds, sched, n_workers=1, batched=False, max_batch=1)
    idx = ReadIndex(ds.reads, len(ds.contigs))
    p = _abi.default_params()
    n_ok = n_var = 0
    for (_, q), a, b in zip(sched, mix, alone):
        rb, re = idx.range_for(q.contig, q.start, q.stop, lens[q.contig])
        rc, bases, changes, vcf = oracle.target(ds.reads, p, ds.names[q.contig], ds.contigs[q.contig], q.contig,
                                                q.start, q.stop, rb, re)
        if rc:
            # a target the reference would crash on fails alone and in the mix
            assert rc == _abi.PG_ERR_INDEX and isinstance(a, IndexError) and isinstance(b, IndexError), q
            continue
        for got in (a, b):
            assert not isinstance(got, Exception), (q, got)
            assert got.fasta == bases, q
            assert got.changes == changes, q
            assert got.vcf == _variant_records(vcf), q
        n_ok += 1
        n_var += changes.count("\n")
    assert n_ok >= len(sched) // 2 and n_var > 0


def test_request_above_the_budget_is_refused(draft):
    from pilon_gb300.engine import EngineError
    ds = draft
    srv = Server(ds.names, ds.contigs, ds.reads, n_workers=1, budget_bytes=1_000_000)
    try:
        big = int(np.argmax([c.size for c in ds.contigs]))
        f = srv.submit(Request(big, 1, int(ds.contigs[big].size)))
        ex = f.exception()
        assert isinstance(ex, EngineError) and ex.status == _abi.PG_ERR_NOMEM
        small = srv.submit(Request(big, 1, 2000)).result()
        assert len(small.fasta) > 0
    finally:
        srv.close()
