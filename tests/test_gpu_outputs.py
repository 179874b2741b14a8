"""End-to-end outputs: FASTA, VCF and changes written through the GB300
engine must be byte-identical to the oracle's restatement of Pilon's writers."""
import os
import tempfile

import numpy as np
import pytest

from oracle import oracle
from pilon_gb300 import _abi, synth
from pilon_gb300.polish import Options, polish

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    from pilon_gb300.engine import Engine
    e = Engine(0)
    yield e
    e.close()


def compare_outputs(engine, ds, params=None, chunk=10_000_000, **kw):
    params = params or _abi.default_params()
    opts = Options(chunk_size=chunk, **kw)
    with tempfile.TemporaryDirectory() as d:
        g = os.path.join(d, "gpu")
        o = os.path.join(d, "ora")
        polish(engine, ds.names, ds.contigs, ds.reads, params, g, opts)
        rc = oracle.polish(ds.reads, params, ds.names, ds.contigs, o, chunk_size=chunk, fix_snps=opts.fix_snps,
                           fix_indels=opts.fix_indels, iupac=opts.iupac, diploid=opts.diploid, vcf_qe=opts.vcf_qe,
                           vcf_date=opts.vcf_date, vcf_source=opts.vcf_source, vcf_args=opts.vcf_args,
                           vcf_ref=opts.vcf_ref)
        assert rc == 0
        for ext in ("fasta", "changes", "vcf"):
            a, b = open(f"{g}.{ext}", "rb").read(), open(f"{o}.{ext}", "rb").read()
            if a != b:
                la, lb = a.split(b"\n"), b.split(b"\n")
                for k, (x, y) in enumerate(zip(la, lb)):
                    if x != y:
                        raise AssertionError(f"{ext} line {k}:\n gpu    {x[:300]!r}\n oracle {y[:300]!r}")
                raise AssertionError(f"{ext}: {len(la)} vs {len(lb)} lines")


def test_outputs_cfg1(engine, cfg1):
    compare_outputs(engine, cfg1)


def test_outputs_cfg1_chunked_options(engine, cfg1):
    compare_outputs(engine, cfg1, chunk=9000, iupac=True, diploid=True)
    compare_outputs(engine, cfg1, params=_abi.default_params(fix_amb=1), chunk=20000, vcf_qe=True)


def test_outputs_many_contigs(engine):
    ds = synth.generate(3, scale=0.01)
    compare_outputs(engine, ds)


def test_outputs_cfg2_scaled(engine):
    ds = synth.generate(2, scale=0.02)
    compare_outputs(engine, ds, chunk=40_000)


def test_outputs_duplication_record(engine):
    # a 14 kb stretch covered twice: copy number 2 -> a <DUP> record
    w = synth.workload(1, scale=1.2)
    ds = synth.generate(w)
    r = ds.reads
    sel = np.nonzero((r.pos > 20_000) & (r.aend < 34_000))[0]
    both = np.sort(np.concatenate([np.arange(r.n_reads), sel]), kind="stable")
    ds.reads = r.subset(both)
    compare_outputs(engine, ds)
