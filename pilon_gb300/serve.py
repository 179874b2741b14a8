"""Serving region-polish requests with continuous batching.

A request is the work of `pilon --targets contig:start-stop --fix snps,indels
--vcf --changes` on one region (S/GenomeFile.scala:215-250 for --targets).
The server is the engine library's own (pg_serve_open / pg_serve_submit /
pg_serve_poll of include/pilon_gb300.h): it keeps the reference and the read
store resident on the device, admits queued requests by the device bytes they
need against a budget, and runs each batch on one of several engine contexts
so that batches overlap on the GPU.  Each answer holds

  fasta    the polished sequence of the region (GenomeRegion.bases after fixIssues)
  changes  the changes-file lines of the region
  vcf      the region's VCF records whose ALT is not "." (a delta)
"""
import ctypes as C
import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass

import numpy as np

from . import _abi
from .polish import Options


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


class Server:
    """The native server of the C ABI (pg_serve_open ... pg_serve_close).

    budget_bytes is the device memory the requests in flight may need together
    (116 bytes per region position and 16 per read of the query window);
    max_batch limits the requests of one batch (0: none); batched=False runs
    each batch on the plain per-region path.  submit() returns a Future of a
    Result, or of an IndexError for a target on which Pilon throws."""

    def __init__(self, names, contigs, reads, params=None, opts=None, n_workers=2, budget_bytes=8 << 30,
                 device=0, batched=True, max_batch=0):
        from .engine import EngineError, lib
        self.L = lib()
        self.opts = opts or Options()
        self.params = params or _abi.default_params()
        cfg = _abi.pg_serve_config()
        self.L.pg_default_serve_config(C.byref(cfg))
        cfg.device, cfg.n_workers, cfg.hbm_budget, cfg.max_batch = device, n_workers, int(budget_bytes), max_batch
        cfg.batched = int(batched)
        cfg.fix_snps, cfg.fix_indels = int(self.opts.fix_snps), int(self.opts.fix_indels)
        cfg.iupac, cfg.diploid, cfg.vcf_qe = int(self.opts.iupac), int(self.opts.diploid), int(self.opts.vcf_qe)
        arrs = [np.ascontiguousarray(c, np.uint8) for c in contigs]
        lens = np.array([a.size for a in arrs], np.int64)
        bases = (C.c_void_p * max(1, len(arrs)))(*[a.ctypes.data for a in arrs])
        nm = [n.encode() for n in names]
        nptr = (C.c_char_p * max(1, len(nm)))(*nm)
        ab = reads.to_abi()
        self.h = C.c_void_p()
        st = self.L.pg_serve_open(C.byref(self.h), C.byref(cfg), C.byref(self.params), len(arrs),
                                  C.cast(nptr, C.c_void_p), lens.ctypes.data, C.cast(bases, C.c_void_p), C.byref(ab))
        if st != 0:
            msg = self.L.pg_serve_error(self.h).decode()
            self.L.pg_serve_close(self.h)
            self.h = None
            raise EngineError(st, msg)
        self._pending = deque()
        self._cv = threading.Condition()
        self._closed = False
        self._poller = threading.Thread(target=self._poll_loop, daemon=True)
        self._poller.start()

    @property
    def batches(self):
        b = C.c_int64()
        self.L.pg_serve_stats(self.h, C.byref(b), None, None)
        return b.value

    def peak_in_flight_bytes(self):
        p = C.c_int64()
        self.L.pg_serve_stats(self.h, None, None, C.byref(p))
        return p.value

    def submit(self, req):
        from .engine import EngineError
        fut = Future()
        q = _abi.pg_request(req.contig, req.start, req.stop, 0)
        t = C.c_uint64()
        st = self.L.pg_serve_submit(self.h, C.byref(q), C.byref(t))
        if st != 0:
            fut.set_exception(EngineError(st, self.L.pg_serve_error(self.h).decode()))
            return fut
        with self._cv:
            self._pending.append((t.value, req, fut))
            self._cv.notify()
        return fut

    def _poll_loop(self):
        from .engine import EngineError
        while True:
            with self._cv:
                while not self._pending and not self._closed:
                    self._cv.wait()
                if not self._pending:
                    return
                t, req, fut = self._pending.popleft()
            res = _abi.pg_result()
            st = self.L.pg_serve_poll(self.h, t, -1, C.byref(res))
            if st != 0:
                fut.set_exception(EngineError(st, self.L.pg_serve_error(self.h).decode()))
                continue
            if res.status == _abi.PG_ERR_INDEX:
                fut.set_exception(IndexError(f"target {req.contig}:{req.start}-{req.stop}: {res.message.decode()}"))
            elif res.status != 0:
                fut.set_exception(EngineError(res.status, res.message.decode()))
            else:
                out = Result(req.rid, C.string_at(res.fasta, res.fasta_len), C.string_at(res.changes,
                             res.changes_len).decode(), C.string_at(res.vcf, res.vcf_len),
                             latency=res.latency_ms / 1e3, batch=res.batch)
                out.queue_ms, out.run_ms, out.device_bytes = res.queue_ms, res.run_ms, res.device_bytes
                fut.set_result(out)
            self.L.pg_serve_release(self.h, t)

    def close(self):
        if self.h is None:
            return
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        self._poller.join()
        self.L.pg_serve_close(self.h)
        self.h = None


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
