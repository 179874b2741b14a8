"""Writes tests/golden/oracle_small.json: digests of the oracle's FASTA, VCF and
changes for a small seeded workload (the 50 kb workload scaled to 10 kb, plus
the same 50 kb workload with 7 kb regions, and 300 kb of the repeat workload
with a gap under --fix all), and per-field array digests of one region.  The reference has no golden files; these pin the oracle against
regressions.  Run: python tests/golden/make_golden.py"""
import hashlib
import json
import os
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from pilon_gb300 import _abi, synth  # noqa: E402


def digests():
    out = {}
    p = _abi.default_params()
    for label, scale, chunk in [("cfg1_10kb", 0.2, 10_000_000), ("cfg1_50kb_chunk7000", 1.0, 7000)]:
        ds = synth.generate(1, scale=scale)
        with tempfile.TemporaryDirectory() as d:
            pre = os.path.join(d, "pilon")
            rc = oracle.polish(ds.reads, p, ds.names, ds.contigs, pre, chunk_size=chunk)
            assert rc == 0
            for ext in ("fasta", "vcf", "changes"):
                out[f"{label}.{ext}"] = hashlib.sha256(open(f"{pre}.{ext}", "rb").read()).hexdigest()
    # --fix snps,indels,gaps,local --K 31 on 300 kb of the repeat workload with a 60 bp gap
    ds = synth.generate(4, scale=0.0025)
    ref = ds.contigs[0].copy()
    ref[150_000:150_060] = ord("N")
    ds.contigs = [ref]
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "pilon")
        assert oracle.polish(ds.reads, p, ds.names, ds.contigs, pre, fix_gaps=True, fix_local=True, K=31) == 0
        for ext in ("fasta", "vcf", "changes"):
            out[f"cfg4_300kb_fix_all.{ext}"] = hashlib.sha256(open(f"{pre}.{ext}", "rb").read()).hexdigest()
        out["cfg4_300kb_fix_all.changes_lines"] = sum(1 for _ in open(pre + ".changes"))
    ds = synth.generate(1, scale=0.2)
    res = oracle.process_region(ds.reads, p, ds.contigs[0], 0, 1, ds.contigs[0].size)
    for f in ["count", "qual_sum", "mq_sum", "q_sum", "phys_cov", "insert_size", "bad_pair", "deletions",
              "insertions", "clips", "call", "score"]:
        out[f"cfg1_10kb.region.{f}"] = hashlib.sha256(getattr(res, f).tobytes()).hexdigest()
    return out


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_small.json")
    json.dump(digests(), open(path, "w"), indent=1, sort_keys=True)
    print(path)
