"""Serving region-polish requests with continuous batching.

A request is the work of `pilon --targets contig:start-stop --fix snps,indels
--vcf --changes` on one region (S/GenomeFile.scala:215-250 for --targets).
The reads of the whole genome stay in device memory once; every worker owns
an engine context (its own CUDA stream and buffers) on the same GPU.  A
worker takes all queued requests that fit its position budget, runs them as
one batched pg_pileup_regions call and answers each with

  fasta    the polished sequence of the region (GenomeRegion.bases after fixIssues)
  changes  the changes-file lines of the region
  vcf      the region's VCF records whose ALT is not "." (a delta)

Requests that arrive while batches run wait only until a worker is free, and
the batches of different workers overlap on the device.
"""
import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass

import numpy as np

from . import _abi
from .polish import Options, _region_outputs, new_name, region_string
from .regions import ReadIndex


@dataclass
class Request:
    contig: int
    start: int
    stop: int
    arrival: float = 0.0
    rid: int = 0


@dataclass
class Result:
    rid: int
    fasta: bytes
    changes: str
    vcf: bytes
    latency: float = 0.0
    batch: int = 0


def device_read_store(reads, device=0):
    """Uploads the read store once (torch tensors as device memory) and returns
    a pg_reads struct of device pointers plus the tensors that own them."""
    import torch
    from .reads import FIELDS
    dev = torch.device(f"cuda:{device}")
    keep = {}
    r = _abi.pg_reads()
    r.n_reads = reads.n_reads
    for f in FIELDS:
        a = np.ascontiguousarray(getattr(reads, f))
        t = torch.from_numpy(a.view(np.uint8).reshape(-1)).to(dev) if a.size else torch.zeros(16, dtype=torch.uint8,
                                                                                             device=dev)
        keep[f] = t
        setattr(r, f, t.data_ptr())
    r.n_cigar_words = int(reads.cigar.size)
    r.seq_bytes = int(reads.seq.size)
    r.qual_bytes = int(reads.qual.size)
    torch.cuda.synchronize(dev)
    return r, keep


def request_result(engine, r, req, names, contigs, params, opts):
    """One region of the last engine call -> the request's answer."""
    region = (req.contig, req.start, req.stop, 0, 0)
    res = _region_outputs(engine, r, region, contigs[req.contig], opts, params)
    nn = new_name(names[req.contig])
    lines = []
    delta = 0
    for f in res.all_fixes():
        nl = f.locus + delta
        lines.append(region_string(names[req.contig], f.locus, f.locus + len(f.was) - 1) + " " +
                     region_string(nn, nl, nl + len(f.patch) - 1) + " " + (f.was or ".") + " " + (f.patch or "."))
        delta += len(f.patch) - len(f.was)
    vcf = engine.format_vcf(r, names[req.contig], opts.diploid, opts.vcf_qe, variants_only=True)
    return Result(req.rid, bytes(res.bases), "".join(l + "\n" for l in lines), vcf)


class Server:
    """Continuous batching over `n_workers` engine contexts on one GPU."""

    def __init__(self, names, contigs, reads, params=None, opts=None, n_workers=2, budget_positions=40_000_000,
                 device=0, batched=True):
        from .engine import Engine
        self.names, self.contigs = names, contigs
        self.params = params or _abi.default_params()
        self.opts = opts or Options()
        self.opts.longread_only = False
        self.opts.vcf = False  # no <DUP> pass for deltas
        self.budget = budget_positions
        self.batched = batched
        self.index = ReadIndex(reads, len(contigs))
        self.dev_reads, self._keep = device_read_store(reads, device)
        self.engines = []
        for _ in range(n_workers):
            e = Engine(device)
            e.set_reference(contigs)
            e.set_reads_device(self.dev_reads, reads.n_reads)
            self.engines.append(e)
        self.q = deque()
        self.cv = threading.Condition()
        self.closed = False
        self.batches = 0
        self.threads = [threading.Thread(target=self._worker, args=(e,), daemon=True) for e in self.engines]
        for t in self.threads:
            t.start()

    def submit(self, req):
        fut = Future()
        if not req.arrival:
            req.arrival = time.perf_counter()
        with self.cv:
            self.q.append((req, fut))
            self.cv.notify()
        return fut

    def _take(self):
        with self.cv:
            while not self.q and not self.closed:
                self.cv.wait()
            if not self.q:
                return []
            batch, used = [], 0
            while self.q:
                req, fut = self.q[0]
                size = req.stop - req.start + 1
                if batch and used + size > self.budget:
                    break
                self.q.popleft()
                batch.append((req, fut))
                used += size
            return batch

    def _worker(self, engine):
        from .engine import EngineError
        while True:
            batch = self._take()
            if not batch:
                return
            try:
                regions = []
                for req, _ in batch:
                    n = int(self.contigs[req.contig].size)
                    a, b = self.index.range_for(req.contig, req.start, req.stop, n)
                    regions.append((req.contig, req.start, req.stop, a, b))
                failed = set()
                try:
                    engine.pileup_regions(regions, self.params, batched=self.batched)
                except EngineError as exc:
                    if exc.status != _abi.PG_ERR_INDEX:
                        raise
                    # the reference throws on these targets; the other requests are unaffected
                    failed = {r for r in range(len(batch)) if engine.stats(r).error}
                with self.cv:
                    self.batches += 1
                    bno = self.batches
                for r, (req, fut) in enumerate(batch):
                    if r in failed:
                        fut.set_exception(IndexError(
                            f"target {self.names[req.contig]}:{req.start}-{req.stop}: an indel left shift leaves "
                            f"the region (Pilon throws ArrayIndexOutOfBoundsException)"))
                        continue
                    out = request_result(engine, r, req, self.names, self.contigs, self.params, self.opts)
                    out.latency = time.perf_counter() - req.arrival
                    out.batch = bno
                    fut.set_result(out)
            except Exception as exc:  # every request of a failed batch sees the error
                for _, fut in batch:
                    if not fut.done():
                        fut.set_exception(exc)

    def close(self):
        with self.cv:
            self.closed = True
            self.cv.notify_all()
        for t in self.threads:
            t.join()
        for e in self.engines:
            e.close()


def poisson_requests(contig_lens, rate, duration, seed=1005, min_len=10_000, max_len=1_000_000):
    """Arrival offsets (s) and regions: Poisson arrivals at `rate`/s, lengths
    log-uniform in [min_len, max_len], clipped to the contig."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t, out = 0.0, []
    lens = np.asarray(contig_lens)
    w = lens / lens.sum()
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        c = int(rng.choice(lens.size, p=w))
        ln = int(np.exp(rng.uniform(np.log(min_len), np.log(max_len))))
        ln = min(ln, int(lens[c]))
        s = int(rng.integers(1, int(lens[c]) - ln + 2))
        out.append((t, Request(c, s, s + ln - 1, rid=len(out))))
    return out


def run_load(server, schedule):
    """Replays `schedule` [(offset_s, Request)] in real time; returns the
    results in request order (an exception object for a failed request) and
    the wall time."""
    t0 = time.perf_counter()
    futs = []
    for off, req in schedule:
        now = time.perf_counter() - t0
        if off > now:
            time.sleep(off - now)
        req.arrival = t0 + off
        futs.append(server.submit(req))
    res = []
    for f in futs:
        exc = f.exception()
        res.append(exc if exc is not None else f.result())
    return res, time.perf_counter() - t0
