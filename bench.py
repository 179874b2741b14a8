"""Benchmark: aligned bases piled per second (pileup + calls + pass 1) on GB300.

Workload (default, --config 3): a draft assembly of 3,000 contigs with
log-normal lengths (median 20 kb, 1 kb - 2 Mb, 132.8 Mb in all), 40x 2x150
pairs, 1% of the bases carrying planted SNPs and indels, synthetic and seeded
(1003); every contig is one region and all 3,000 run as one batched,
graph-replayed plan.  A step is one pg_pileup_regions call over all regions:
BamFile.process + PileUpRegion.addRead, computePhysCov, BaseCall and pass 1.
The line also carries the 5 Mb / 100x bacterial workload (--config 2) measured
the same way under "bacterial_5mb", and "parity_full": every region of the
full-size workload compared with the oracle (outside the timed region), and
"polish_driver": the whole polishing run (--fix snps,indels, FASTA and changes)
on the workload, host wall clock.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config 3] [--impl reference]

--impl reference times the CPU restatement of the reference path (the oracle;
the Scala reference cannot run here: no JVM) on the host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gbases piled/s (aligned M/=/X bases walked per region, pileup+calls+pass 1)"
UNIT = "Gbases/s"


def piled_bases(reads, regions, contig_lens, params):
    """Iterations of the M/=/X loop of PileUpRegion.addRead (S/PileUpRegion.scala:184-193)
    summed over the reads fed to each region (validated reads in the query window)."""
    m = reads.aligned_bases()
    fl = reads.flag.astype(np.int64)
    ok = np.ones(reads.n_reads, bool)
    if not params.nonpf:
        ok &= (fl & 0x200) == 0
    if not params.duplicates:
        ok &= (fl & 0x400) == 0
    ok &= (fl & 0x100) == 0
    tot = 0
    for (c, s, e, rb, re) in regions:
        qs, qe = max(s - 10000, 0), min(e + 10000, int(contig_lens[c]))
        pos = reads.pos[rb:re].astype(np.int64)
        end = np.where((fl[rb:re] & 4) != 0, pos, reads.aend[rb:re].astype(np.int64))
        sel = ok[rb:re] & (reads.ref_id[rb:re] == c) & (pos <= qe) & (end >= qs)
        tot += int(m[rb:re][sel].sum())
    return tot


def walk_algorithmic_bytes(reads, regions):
    """Bytes the walk must move at minimum: per read fed to a region its header
    (32 B), CIGAR (4 B/op), 2-bit bases (L/4) and qualities (L), plus the
    88-byte pileup record written once per position."""
    L = reads.l_seq.astype(np.int64)
    per_read = 32 + 4 * reads.n_cigar.astype(np.int64) + (L + 3) // 4 + L
    csum = np.concatenate([[0], np.cumsum(per_read)])
    b = 0
    for (c, s, e, rb, re) in regions:
        b += int(csum[re] - csum[rb]) + 88 * (e - s + 1)
    return b


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "20"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.p:
            self.p.terminate()
            try:
                out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# the fields pg_set_reads_packed derives on the device instead of uploading
PACKED_DERIVED = ("aend", "cigar_off", "seq_off", "qual_off")


def pinned_store(reads, packed=False):
    """Copies the read store into page-locked host memory (torch pinned tensors);
    packed=True leaves out the fields the packed upload derives on the device."""
    import torch
    from pilon_gb300.reads import FIELDS, ReadStore
    keep = []
    arrs = {}
    for f in FIELDS:
        a = np.ascontiguousarray(getattr(reads, f))
        if packed and f in PACKED_DERIVED:
            arrs[f] = np.zeros(0, a.dtype)
            continue
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        v = t.numpy().view(a.dtype)
        v[:] = a.reshape(-1)
        keep.append(t)
        arrs[f] = v
    st = ReadStore(**arrs)
    st._pinned = keep
    return st


class PinnedOut:
    CALL_FIELDS = ("call", "score", "indel_len", "ins_str")

    def __init__(self, size, fields="all"):
        import torch
        from pilon_gb300.engine import RegionArrays
        self.t = []
        ra = RegionArrays.__new__(RegionArrays)
        ra.size = size

        def mk(n, dt):
            t = torch.empty(n * np.dtype(dt).itemsize, dtype=torch.uint8, pin_memory=True)
            self.t.append(t)
            return t.numpy().view(dt)
        want = lambda f: fields == "all" or f in self.CALL_FIELDS
        ra.count = mk(4 * size, np.int32) if want("count") else None
        ra.qual_sum = mk(4 * size, np.int64) if want("qual_sum") else None
        for f in RegionArrays.I32:
            setattr(ra, f, mk(size, np.int32) if want(f) else None)
        ra.call = mk(size, np.uint32)
        ra.score = mk(size, np.int64)
        ra.ins_chars = np.zeros(0, np.uint8)
        self.arrays = ra

    def nbytes(self):
        return sum(t.numel() for t in self.t)


def roofline_traffic(workload_name, units):
    """Per-launch DRAM bytes of the walk kernel from the committed ncu summary:
    the capture of this workload's scaled-down case (lines tagged with the
    workload name) or else the untagged one, scaled by units (piled bases),
    since the walk's DRAM bytes grow with the reads it walks; None if absent."""
    path = os.path.join(ROOT, "profiles", "k_walk_ncu.md")
    if not os.path.exists(path):
        return None
    found = {}
    for line in open(path):
        for key in ("traffic_bytes_per_launch", "units_per_launch"):
            if line.startswith(key):
                tag = line[len(key):line.index(":")].strip("[] ")
                found[(key, tag)] = float(line.split(":")[1])
    for tag in (workload_name, ""):
        b, u = found.get(("traffic_bytes_per_launch", tag)), found.get(("units_per_launch", tag))
        if b is not None:
            return b * units / u if u else b
    return None


def oracle_sample(ds, params, threads, regions=None):
    """The oracle over the whole workload on `threads` host threads: on the
    GPU arm's own regions when there are at least as many as threads (then both
    arms pile the same units), else with each contig split in up to `threads`
    regions; largest regions first.  Returns (piled bases, seconds, regions)."""
    from oracle import oracle
    from pilon_gb300.regions import ReadIndex
    oracle.lib()
    if regions is not None and len(regions) >= threads:
        jobs = sorted(regions, key=lambda r: r[1] - r[2])
    else:
        jobs = []
        idx = ReadIndex(ds.reads, len(ds.contigs))
        for ci, ref in enumerate(ds.contigs):
            n = max(1, min(threads, ref.size // 50_000))
            step = (ref.size + n - 1) // n
            for s in range(1, ref.size + 1, step):
                e = min(ref.size, s + step - 1)
                a, b = idx.range_for(ci, s, e, ref.size)
                jobs.append((ci, s, e, a, b))
    units = piled_bases(ds.reads, jobs, [c.size for c in ds.contigs], params)
    res = [None] * len(jobs)
    it = iter(range(len(jobs)))
    lock = threading.Lock()

    def worker():
        while True:
            with lock:
                k = next(it, None)
            if k is None:
                return
            ci, s, e, a, b = jobs[k]
            res[k] = oracle.process_region(ds.reads, params, ds.contigs[ci], ci, s, e, a, b).status
    t0 = time.perf_counter()
    ths = [threading.Thread(target=worker) for _ in range(threads)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    return units, time.perf_counter() - t0, len(jobs)


def kmer_bench(eng, ds, params, args, threads, K=31, radius=500):
    """120 Mb genome with repeats: the K-mer tally of Assembler.addReads/buildGraph (pg_kmer_tally)
    over one local-reassembly window per planted indel (the reads overlapping
    [x - 500, x + 500]), on the GPU and on the oracle over all host threads for
    a sample of windows, with the sample's edges compared."""
    from oracle import oracle
    from pilon_gb300.regions import ReadIndex
    idx = ReadIndex(ds.reads, len(ds.contigs))
    wins = []
    for ci, var in enumerate(ds.variants):
        n = ds.contigs[ci].size
        for v in var:
            wins.append(idx.range_for(ci, max(1, v[0] - radius), min(n, v[0] + radius), n, slop=0))
    L = ds.reads.l_seq.astype(np.int64)
    per = np.concatenate([[0], np.cumsum(2 * np.maximum(L - K, 0))])
    events = int(sum(per[b] - per[a] for a, b in wins))
    for _ in range(args.warmup):
        edges = eng.kmer_tally(wins, K, params)
    t = []
    for _ in range(max(3, min(args.steps, 10))):
        t0 = time.perf_counter()
        edges = eng.kmer_tally(wins, K, params)
        t.append(time.perf_counter() - t0)
    sec = sum(t) / len(t)
    dev_ms, dev_events, distinct, batch_bytes, batches = eng.last_tally_stats()
    # algorithmic bytes: every window read once (2-bit bases, qualities and 16 B of
    # offsets, length and mapq), then per distinct K-mer its 8-byte key and the
    # PileUp fields buildGraph reads (4 counts, 4 Long quality sums, qSum: 52 B)
    # written once
    rb = np.concatenate([[0], np.cumsum((L + 3) // 4 + L + 16)])
    read_bytes = int(sum(rb[b] - rb[a] for a, b in wins))
    tally_bytes = read_bytes + 60 * distinct
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    hbm = peaks["hbm_gbs"] if peaks else 6800.0
    device = {"ms": dev_ms, "value": dev_events / (dev_ms / 1e3) / 1e9, "unit": "G K-mer events/s",
              "kmer_events": dev_events, "distinct_kmers": distinct, "batches": batches,
              "max_batch_table_bytes": batch_bytes, "l2_bytes": 129 * 2**20,
              "tables_within_l2": batch_bytes <= 129 * 2**20,
              "roofline": {"bound": "hbm", "achieved": tally_bytes / (dev_ms / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                           "frac": tally_bytes / (dev_ms / 1e3) / 1e9 / hbm, "algorithmic_bytes": tally_bytes,
                           "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback"},
              "timing": "CUDA events around the tally kernels on the engine stream (pg_last_tally_stats)"}
    # the same tally over one window per device break candidate, built on the device
    eng.pileup_regions(ds_regions(ds), params, batched=True)
    tb = []
    for _ in range(3):
        t0 = time.perf_counter()
        nwb, eb = eng.kmer_tally_breaks(K, params, radius=radius)
        tb.append(time.perf_counter() - t0)
    from_breaks = {"windows": nwb, "edges": int(len(eb)), "ms_per_call": 1e3 * min(tb),
                   "timing": "host wall clock of pg_kmer_tally_breaks (windows built on the device)"}
    out = {"windows": len(wins), "K": K, "kmer_events": events, "edges": int(len(edges)),
           "ms_per_call": 1e3 * sec, "value": events / sec / 1e9, "unit": "G K-mer events/s",
           "timing": "host wall clock of pg_kmer_tally, edges read back", "device": device,
           "from_device_breaks": from_breaks}
    if not args.no_cpu:
        sample = wins[: max(1, min(len(wins), 16 * threads))]
        parts = [sample[k::threads] for k in range(threads)]
        res = [None] * threads

        def worker(k):
            res[k] = oracle.kmer_tally(ds.reads, params, parts[k], K) if parts[k] else None
        t0 = time.perf_counter()
        ths = [threading.Thread(target=worker, args=(k,)) for k in range(threads)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        csec = time.perf_counter() - t0
        sev = int(sum(per[b] - per[a] for a, b in sample))
        # the GPU edges of the sampled windows, against the oracle's
        got = eng.kmer_tally(sample, K, params)

        def edge_set(e, remap):
            return {(remap(int(x["window"])), int(x["key_hi"]), int(x["key_lo"]), int(x["next"]), int(x["alt"]),
                     int(x["depth"]), int(x["weight"])) for x in e}
        want = set()
        for k in range(threads):
            if res[k] is not None:
                want |= edge_set(res[k], lambda w, k=k: k + threads * w)
        out["cpu_baseline"] = {"value": sev / csec / 1e9, "unit": "G K-mer events/s", "cores": threads,
                               "kind": "port", "sample": f"{len(sample)} of {len(wins)} windows on {threads} host "
                                                         f"threads"}
        out["sample_edges_identical"] = edge_set(got, lambda w: w) == want
    return out


def fix_all_bench(eng, ds, params, K=31):
    """--fix snps,indels,gaps,local over the whole 120 Mb workload through the
    polishing driver (FASTA and changes written, no VCF), against the same run
    with --fix snps,indels: the local-reassembly steps' times (scan and
    recruitment on the host, the K-mer tally of every window on the device,
    the graph walks on host threads) and counts."""
    import tempfile
    from pilon_gb300.polish import Options, polish
    out = {"K": K, "timing": "host wall clock of polish(); the reassembly steps timed inside it"}
    with tempfile.TemporaryDirectory() as d:
        for key, kw in (("snps_indels", {}), ("all", dict(fix_gaps=True, fix_local=True, K=K))):
            opts = Options(vcf=False, **kw)
            opts.stats = {}
            t0 = time.perf_counter()
            polish(eng, ds.names, ds.contigs, ds.reads, params, os.path.join(d, key), opts)
            out[key + "_s"] = time.perf_counter() - t0
            if opts.stats:
                out["reassembly"] = opts.stats
        out["changes_lines"] = sum(1 for _ in open(os.path.join(d, "all.changes")))
    return out


def polish_bench(eng, ds, params, reps=2):
    """The whole polishing driver on the workload, --fix snps,indels with the
    FASTA and changes written (no VCF): reference and read store upload,
    pg_pileup_regions, the change list, the fix lists, fixIssues and the
    writers, as Pilon's processRegions runs them.  Host wall clock; the
    engine calls' share timed inside it."""
    import tempfile
    from pilon_gb300.polish import Options, polish
    calls = {}

    class Timed:  # the engine, with the time of each call polish() makes summed by name
        def __init__(self, inner):
            self._inner = inner

        def __getattr__(self, name):
            f = getattr(self._inner, name)
            if not callable(f):
                return f

            def g(*a, **k):
                t = time.perf_counter()
                try:
                    return f(*a, **k)
                finally:
                    calls[name] = calls.get(name, 0.0) + time.perf_counter() - t
            return g

    runs = []
    with tempfile.TemporaryDirectory() as d:
        for _ in range(reps):
            calls.clear()
            t0 = time.perf_counter()
            polish(Timed(eng), ds.names, ds.contigs, ds.reads, params, os.path.join(d, "o"), Options(vcf=False))
            runs.append((time.perf_counter() - t0, dict(calls)))
        lines = sum(1 for _ in open(os.path.join(d, "o.changes")))
        fasta = os.path.getsize(os.path.join(d, "o.fasta"))
    best, engine_calls = min(runs, key=lambda x: x[0])
    return {"seconds": best, "runs_s": [r[0] for r in runs], "engine_calls_s": engine_calls,
            "changes_lines": lines, "fasta_bytes": fasta, "fix": "snps,indels", "outputs": "FASTA, changes",
            "timing": "host wall clock of polish(), the best of the runs; engine_calls_s sums the engine calls "
                      "it makes (uploads, pileup, change list, region statistics)"}


def extra_workload(config, args, params, device, peak, peaks):
    """A second workload on its own engine context: device-timed steps (CUDA
    events, after warm-up) and the walk kernel's roofline, as for the main one."""
    from pilon_gb300 import synth
    from pilon_gb300.engine import Engine
    from pilon_gb300.regions import plan_regions
    ds = synth.generate(config, args.scale)
    lens = [c.size for c in ds.contigs]
    regions = plan_regions(ds.reads, lens)
    units = piled_bases(ds.reads, regions, lens, params)
    walk_bytes = walk_algorithmic_bytes(ds.reads, regions)
    eng = Engine(device)
    try:
        eng.set_reference(ds.contigs)
        eng.set_reads(ds.reads)
        from pilon_gb300.autotune import tune
        best, _ = tune(eng, regions, params, f"{ds.workload.name}:{args.scale}:1", batched=True)
        for _ in range(args.warmup):
            eng.pileup_regions(regions, params, batched=True)
        eng.sync()
        tot, walk = [], []
        for _ in range(max(3, min(args.steps, 20))):
            eng.pileup_regions(regions, params, batched=True)
            w, t, _ = eng.last_kernel_ms()
            tot.append(t)
            walk.append(w)
        eng.sync()
    finally:
        eng.close()
    walk_s = sum(walk) / len(walk) / 1e3
    achieved = walk_bytes / walk_s / 1e9
    return {"key": "bacterial_5mb" if config == 2 else f"workload_{config}", "workload": ds.workload.name,
            "value": units * len(tot) / (sum(tot) / 1e3) / 1e9, "unit": UNIT, "ms_per_step": sum(tot) / len(tot),
            "piled_bases_per_step": units, "steps": len(tot),
            "tuning": {"tile_width": best[0], "warps": best[1], "variant": best[2]},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": roofline_traffic(ds.workload.name, units), "kernel": "k_walk",
                         "algorithmic_bytes_per_launch": walk_bytes, "walk_ms": walk_s * 1e3,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback"},
            "timing": "CUDA events on the engine stream, inputs resident in HBM (larger than L2)"}


def ds_regions(ds):
    from pilon_gb300.regions import plan_regions
    return plan_regions(ds.reads, [c.size for c in ds.contigs])


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
        return dist, int(os.environ["RANK"]), ws, int(os.environ.get("LOCAL_RANK", "0"))
    return None, 0, 1, 0


def barrier(dist):
    if dist:
        dist.barrier()


def max_over_ranks(dist, v):
    if not dist:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def serve_bench(args, dist, rank, ws, local, params):
    """Serving through the C ABI (pg_serve_*): Poisson arrivals (lambda = 200/s)
    of region-polish requests of 10 kb - 1 Mb (log-uniform) against the
    device-resident read store of the many-contig workload; continuous batching
    admitted by device bytes vs the plain path (one request per batch,
    per-region launches), then the same at a rate that saturates the plain
    path, for the throughput of both."""
    from pilon_gb300 import synth
    from pilon_gb300.serve import Server, poisson_requests, run_load
    ds = synth.generate(3, args.scale)
    lens = [c.size for c in ds.contigs]
    m = ds.reads.aligned_bases()
    from pilon_gb300.regions import ReadIndex
    idx = ReadIndex(ds.reads, len(ds.contigs))

    def summary(sched, res, wall, label, batches):
        ok = [r for r in res if not isinstance(r, Exception)]
        lat = np.array([r.latency for r in ok]) * 1e3
        units = 0
        for _, q in sched:
            a, b = idx.range_for(q.contig, q.start, q.stop, lens[q.contig])
            units += int(m[a:b].sum())
        return {"path": label, "requests": len(res), "failed_like_reference": len(res) - len(ok),
                "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                "throughput_req_s": len(res) / wall, "gbases_per_s": units / wall / 1e9, "wall_s": wall,
                "batches": batches}

    def run(rate, duration, batched_path):
        sched = poisson_requests(lens, rate=rate, duration=duration)
        kw = dict(n_workers=args.workers, budget_bytes=args.budget) if batched_path else \
            dict(n_workers=1, batched=False, max_batch=1)
        srv = Server(ds.names, ds.contigs, ds.reads, params, device=local, **kw)
        try:
            run_load(srv, poisson_requests(lens, rate=rate, duration=min(1.0, duration), seed=99))  # warm-up
            b0 = srv.batches
            res, wall = run_load(srv, sched)
            label = (f"continuous batching, {args.workers} contexts, {args.budget / 2**30:.1f} GiB budget"
                     if batched_path else "one request per batch, per-region launches")
            out = summary(sched, res, wall, label, srv.batches - b0)
            if batched_path:
                out["peak_in_flight_bytes"] = srv.peak_in_flight_bytes()
            return out, res
        finally:
            srv.close()

    out = {}
    out["batched"], res = run(args.rate, args.duration, True)
    out["plain"], pres = run(args.rate, args.duration, False)
    same = all((isinstance(a, Exception) and isinstance(b, Exception)) or
               (not isinstance(a, Exception) and not isinstance(b, Exception) and a.fasta == b.fasta and
                a.changes == b.changes and a.vcf == b.vcf) for a, b in zip(res, pres))
    sat = None
    if args.saturate_rate > 0:
        sb, _ = run(args.saturate_rate, args.saturate_duration, True)
        sp, _ = run(args.saturate_rate, args.saturate_duration, False)
        sat = {"rate_per_s": args.saturate_rate, "duration_s": args.saturate_duration, "batched": sb, "plain": sp,
               "throughput_batched_over_plain": sb["throughput_req_s"] / sp["throughput_req_s"]}
    if rank != 0:
        return
    b = out["batched"]
    line = {"metric": "served-region latency p99 (ms) at lambda = %g/s" % args.rate, "value": b["p99_ms"],
            "unit": "ms", "higher_is_better": False, "n_gpus": ws, "steps": b["requests"], "warmup": 1,
            "ms_per_step": b["mean_ms"], "scaling": "weak", "vs_baseline": None, "dtype": "int32/int64",
            "data": "synthetic (seeded)", "config": {"workload": "serving over draft-3000-contigs-40x",
            "genome_bp": int(sum(lens)), "reads": ds.reads.n_reads, "rate_per_s": args.rate,
            "duration_s": args.duration, "request_bp": "10 kb - 1 Mb log-uniform"},
            "served": out, "identical_outputs_batched_vs_plain": same, "saturated": sat,
            "path": "C ABI server (pg_serve_submit / pg_serve_poll), latency from submit to answer"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", type=int, default=3)
    ap.add_argument("--extra-config", type=int, default=-1, help="a second workload measured the same way "
                    "(device-timed steps and the walk roofline); default 2 when --config is 3, 0 = none")
    ap.add_argument("--no-parity", action="store_true", help="skip the full-size comparison with the oracle")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--batched", type=int, default=1)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--warps", type=int, default=0)
    ap.add_argument("--variant", type=int, default=-1)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--compare-plain", type=int, default=-1, help="also time the per-region path (default: on "
                    "when there is more than one region)")
    ap.add_argument("--e2e-fields", default="auto", help="changes (default) | all | calls: what the end-to-end "
                    "step reads back")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: requests per second")
    ap.add_argument("--duration", type=float, default=10.0, help="serving: seconds of arrivals")
    ap.add_argument("--workers", type=int, default=2, help="serving: engine contexts")
    ap.add_argument("--budget", type=float, default=float(8 << 30), help="serving: device bytes in flight")
    ap.add_argument("--saturate-rate", type=float, default=1500.0, help="serving: a rate that saturates the "
                    "plain path (0 = skip)")
    ap.add_argument("--saturate-duration", type=float, default=3.0)
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    dist, rank, ws, local = dist_init()
    from pilon_gb300 import _abi, synth
    from pilon_gb300.regions import plan_regions

    params = _abi.default_params()
    threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()

    if args.impl == "reference":
        if rank != 0:
            return
        ds = synth.generate(args.config, args.scale)
        ref_regions = plan_regions(ds.reads, [c.size for c in ds.contigs])
        samples = []
        for k in range(args.warmup + args.steps):
            units, sec, njobs = oracle_sample(ds, params, threads, ref_regions)
            if k >= args.warmup:
                samples.append((units, sec))
        units = sum(u for u, _ in samples)
        sec = sum(s for _, s in samples)
        v = units / sec / 1e9
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / len(samples),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32/int64",
                "data": "synthetic (seeded)",
                "config": {"workload": ds.workload.name, "genome_bp": int(sum(c.size for c in ds.contigs)),
                           "reads": ds.reads.n_reads, "coverage": ds.workload.coverage},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": f"whole workload per step, split into {njobs} regions over {threads} "
                                           f"host threads (the Scala reference needs a JVM, absent here)"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if args.config == 5:
        return serve_bench(args, dist, rank, ws, local, params)

    from pilon_gb300.engine import Engine
    ds = synth.generate(args.config, args.scale)
    lens = [c.size for c in ds.contigs]
    regions = plan_regions(ds.reads, lens)
    units = piled_bases(ds.reads, regions, lens, params)
    walk_bytes = walk_algorithmic_bytes(ds.reads, regions)

    eng = Engine(local)
    if args.tile or args.warps or args.variant >= 0:
        eng.set_tuning(args.tile, args.warps, args.variant)
    eng.set_reference(ds.contigs)
    eng.set_reads(ds.reads)
    tuning = None
    if args.autotune and not (args.tile or args.warps or args.variant >= 0):
        from pilon_gb300.autotune import tune
        best, table = tune(eng, regions, params, f"{ds.workload.name}:{args.scale}:{int(args.batched)}",
                           batched=bool(args.batched))
        tuning = {"tile_width": best[0], "warps": best[1], "variant": best[2], "walk_ms": best[3],
                  "table": table}
    clk = ClockSampler(local)
    clk.__enter__()  # sampled from warm-up start to the end of the timed region
    time.sleep(0.3)  # let nvidia-smi start sampling
    for _ in range(args.warmup):
        eng.pileup_regions(regions, params, batched=bool(args.batched))
    barrier(dist)
    eng.sync()
    tot_ms, walk_ms, launches = [], [], 0
    for _ in range(args.steps):
        eng.pileup_regions(regions, params, batched=bool(args.batched))
        w, t, n = eng.last_kernel_ms()
        tot_ms.append(t)
        walk_ms.append(w)
        launches += n
    eng.sync()
    clk.__exit__()
    barrier(dist)
    dev_s = max_over_ranks(dist, sum(tot_ms) / 1e3)
    value = units * ws * args.steps / dev_s / 1e9
    walk_avg = sum(walk_ms) / len(walk_ms) / 1e3
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = walk_bytes / walk_avg / 1e9
    traffic = roofline_traffic(ds.workload.name, units)

    # the plain path: every region through its own launches, no graph
    plain = None
    if (args.compare_plain == 1 or (args.compare_plain == -1 and len(regions) > 1)) and args.batched:
        for _ in range(2):
            eng.pileup_regions(regions, params, batched=False)
        pm, pn = [], 0
        for _ in range(max(2, min(args.steps, 5))):
            eng.pileup_regions(regions, params, batched=False)
            w, t, n = eng.last_kernel_ms()
            pm.append(t)
            pn = n
        ps = max_over_ranks(dist, sum(pm) / 1e3)
        plain = {"value": units * ws * len(pm) / ps / 1e9, "ms_per_step": 1e3 * ps / len(pm),
                 "gpu_launches_per_step": pn, "path": "one set of launches per region, no graph"}
        eng.pileup_regions(regions, params, batched=True)

    # break candidates of every region on the device (pg_find_breaks), after a batched call
    bt, n_breaks = [], 0
    for _ in range(3):
        eng.pileup_regions(regions, params, batched=bool(args.batched))  # breaks are found once per call
        eng.sync()
        t0 = time.perf_counter()
        br = eng.find_breaks(params.min_min_depth)
        bt.append(time.perf_counter() - t0)
        n_breaks = sum(len(v) for v in br.values())
    breaks = {"ms_per_call": 1e3 * min(bt), "breaks": n_breaks, "positions": int(sum(e - s + 1 for (c, s, e, a, b) in regions)),
              "timing": "host wall clock of pg_find_breaks (device kernels, sorted list read back)"}

    # end to end through the C ABI: H2D of the read store from pinned memory,
    # pileup + calls, D2H of the step's result: by default the pass-1 changes of
    # every region with their insertion strings (pg_fetch_changes, what the fix
    # lists, FASTA and changes file are made from), or with --e2e-fields all |
    # calls every position's records / calls.  Measured with one engine context
    # (each step's calls wait for the previous step's) and with two contexts on
    # two host threads, the way a host serves several requests: one context's
    # read-back overlaps the other's upload.
    e2e = None
    if not args.no_e2e:
        fields = args.e2e_fields if args.e2e_fields != "auto" else "changes"
        # the store is packed (each read's CIGAR, bases and qualities after the
        # previous read's), so its offsets and alignment ends are derived on the
        # device (pg_set_reads_packed) and only the other fields are uploaded
        pin = pinned_store(ds.reads, packed=True)
        n_pos = sum(e - s + 1 for (c, s, e, a, b) in regions)
        outs = [PinnedOut(n_pos, fields) if fields != "changes" else None]  # all regions, one after another
        h2d = pin.nbytes()
        if fields == "changes":
            eng.pileup_regions(regions, params, batched=bool(args.batched))
            ch, chars = eng.fetch_changes()
            d2h = ch.nbytes + len(chars)
        else:
            d2h = outs[0].nbytes()

        def e2e_step(e, o):
            e.set_reads(pin, packed=True)
            e.pileup_regions(regions, params, batched=bool(args.batched))
            if o is None:
                e.fetch_changes()
            else:
                e.fetch_all(o.arrays)

        for _ in range(args.warmup):
            e2e_step(eng, outs[0])
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step(eng, outs[0])
        eng.sync()
        one_s = max_over_ranks(dist, time.perf_counter() - t0)
        barrier(dist)

        shape = (tuning["tile_width"], tuning["warps"], tuning["variant"]) if tuning else \
            (args.tile, args.warps, args.variant)
        eng2 = Engine(local)
        eng2.set_tuning(*shape)
        eng2.set_reference(ds.contigs)
        outs.append(PinnedOut(n_pos, fields) if fields != "changes" else None)
        engines = [eng, eng2]
        for _ in range(args.warmup):
            e2e_step(eng2, outs[1])
        import threading
        counts = [(args.steps + 1) // 2, args.steps // 2]
        errs = []

        def worker(k):
            try:
                for _ in range(counts[k]):
                    e2e_step(engines[k], outs[k])
                engines[k].sync()
            except Exception as ex:  # reported after the join
                errs.append(ex)

        barrier(dist)
        t0 = time.perf_counter()
        ths = [threading.Thread(target=worker, args=(k,)) for k in range(2)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        two_s = max_over_ranks(dist, time.perf_counter() - t0)
        barrier(dist)
        eng2.close()
        if errs:
            raise errs[0]
        e2e = {"value": units * ws * args.steps / two_s / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * two_s / args.steps, "read_back": fields,
               "contexts": 2,
               "one_context": {"value": units * ws * args.steps / one_s / 1e9, "ms_per_step": 1e3 * one_s / args.steps},
               "timing": "host wall clock; every call synchronises its context's stream; two contexts on two "
                         "host threads take alternate steps"}

    kmer = kmer_bench(eng, ds, params, args, threads) if args.config == 4 and rank == 0 else None
    if kmer is not None:
        kmer["fix_all"] = fix_all_bench(eng, ds, params)

    # BAM decoding into the read store (the htsjdk side of BamFile), host threads
    bam_decode = None
    if args.config in (1, 2) and rank == 0 and not args.no_cpu:
        import tempfile
        from pilon_gb300 import bam
        try:  # a failure of the host decoder is reported in the line, not fatal to it
            with tempfile.TemporaryDirectory() as d:
                path = os.path.join(d, "reads.bam")
                bam.write_bam(path, ds.names, lens, ds.reads, threads=threads)
                size = os.path.getsize(path)
                bt2 = []
                for _ in range(2):
                    t0 = time.perf_counter()
                    _, _, st = bam.read_bam(path, threads=threads)
                    bt2.append(time.perf_counter() - t0)
                same = all(np.array_equal(getattr(st, f), getattr(ds.reads, f)) for f in ("pos", "cigar", "seq", "qual"))
            bam_decode = {"reads_per_s": ds.reads.n_reads / min(bt2), "compressed_MB_per_s": size / min(bt2) / 1e6,
                          "file_MB": size / 1e6, "threads": threads, "store_identical": same,
                          "timing": "host wall clock of bam.read_bam: BGZF inflate (own DEFLATE decoder) and "
                                    "record split on native threads"}
        except Exception as ex:  # noqa: BLE001
            bam_decode = {"error": f"{type(ex).__name__}: {ex}"}

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu:
        u, sec, njobs = oracle_sample(ds, params, threads, regions)
        same = njobs == len(regions) and u == units
        cpu = {"value": u / sec / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": (f"the whole workload on the GPU arm's {njobs} regions" if same else
                          f"the whole workload split into {njobs} regions") + f" on {threads} host threads, one pass",
               "same_units_as_gpu": same}
        if not args.no_parity:
            # every region of the full-size workload against the oracle,
            # outside the timed region
            from oracle.parity import full_parity
            t0 = time.perf_counter()
            try:
                n_reg, n_pos = full_parity(eng, ds, params, regions, threads, batched=bool(args.batched))
                parity = {"identical": True, "regions": n_reg, "positions": n_pos}
            except AssertionError as ex:
                parity = {"identical": False, "first_difference": str(ex)[:300]}
            parity.update({"workload": ds.workload.name, "path": "batched" if args.batched else "per-region",
                           "compared": "every pileup counter, call flag, score, indel length and string and "
                                       "region statistic of every region, bit for bit",
                           "seconds": time.perf_counter() - t0})
    driver = None
    if args.config in (1, 2, 3) and rank == 0:
        try:  # a failure of the host driver is reported in the line, not fatal to it
            driver = polish_bench(eng, ds, params)
        except Exception as ex:  # noqa: BLE001
            driver = {"error": f"{type(ex).__name__}: {ex}"[:300]}
    extra = None
    xc = args.extra_config if args.extra_config >= 0 else (2 if args.config == 3 else 0)
    if xc and xc != args.config and rank == 0:
        extra = extra_workload(xc, args, params, local, peak, peaks)
    eng.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32/int64", "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": ds.workload.name, "genome_bp": int(sum(lens)), "regions": len(regions),
                   "reads": ds.reads.n_reads, "coverage": ds.workload.coverage, "piled_bases_per_step": units,
                   "path": "batched" if args.batched else "per-region", "l2": "inputs larger than L2 (reads "
                   f"{ds.reads.nbytes() / 1e6:.0f} MB)", "parallelism": f"replicas x{ws}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": "k_walk", "algorithmic_bytes_per_launch": walk_bytes,
                     "walk_ms": walk_avg * 1e3, "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"
                     if peaks else "fallback"},
        "gpu_launches": launches,
        "tuning": tuning,
        "plain_per_region": plain,
        "batched_over_plain": (value / plain["value"]) if plain else None,
        "clocks": clk.summary(),
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    line["break_candidates"] = breaks
    if parity:
        line["parity_full"] = parity
    if extra:
        line[extra.pop("key")] = extra
    if bam_decode:
        line["bam_decode"] = bam_decode
    if kmer:
        line["kmer_tally"] = kmer
    if driver:
        line["polish_driver"] = driver
    print(json.dumps(line))


if __name__ == "__main__":
    main()
