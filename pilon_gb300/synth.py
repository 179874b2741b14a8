"""Seeded synthetic genomes and read sets for the five benchmark workloads.

No public dataset is used; every input is generated here from a fixed seed
per workload (1001-1005): a random reference, planted SNPs and indels in
a sample copy of it, and paired 2x150 reads drawn from the sample with CIGARs
from their true alignment to the reference.  The per-read simulation runs in
libpg_synth.so (C++); reference and variant planting use numpy PCG64.
"""
import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from .reads import ReadStore, concat_stores

_SYNTH = None


def _lib():
    global _SYNTH
    if _SYNTH is None:
        from .build import SYNTH, build
        if not os.path.exists(SYNTH):
            build()
        _SYNTH = C.CDLL(SYNTH)
        _SYNTH.sy_simulate.restype = C.c_void_p
        _SYNTH.sy_simulate.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                       C.c_uint64]
        _SYNTH.sy_n_reads.restype = C.c_int64
        _SYNTH.sy_n_reads.argtypes = [C.c_void_p]
        _SYNTH.sy_n_cigar.restype = C.c_int64
        _SYNTH.sy_n_cigar.argtypes = [C.c_void_p]
        _SYNTH.sy_copy.argtypes = [C.c_void_p] + [C.c_void_p] * 14
        _SYNTH.sy_copy_pairs.argtypes = [C.c_void_p, C.c_void_p]
        _SYNTH.sy_free.argtypes = [C.c_void_p]
    return _SYNTH


class _SimParams(C.Structure):
    _fields_ = [("read_len", C.c_int32), ("coverage", C.c_double), ("insert_mean", C.c_double),
                ("insert_sd", C.c_double), ("sub_err", C.c_double), ("indel_err", C.c_double),
                ("n_frac", C.c_double), ("mapq0_frac", C.c_double), ("clip_frac", C.c_double),
                ("dup_frac", C.c_double), ("secondary_frac", C.c_double), ("improper_frac", C.c_double),
                ("noqual_frac", C.c_double), ("ref_id", C.c_int32), ("repeat_mapq_max", C.c_int32)]


@dataclass
class Workload:
    name: str
    seed: int
    contig_lengths: list
    gc: float = 0.5
    coverage: float = 50.0
    read_len: int = 150
    insert_mean: float = 400.0
    insert_sd: float = 50.0
    n_snps: int = 20             # per whole genome (spread over contigs by length)
    n_indels: int = 5
    indel_len: tuple = (1, 10)
    variant_frac: float = 0.0    # if > 0: fraction of bases carrying planted variants
    sub_err: float = 0.005
    indel_err: float = 0.0
    n_frac: float = 1e-4
    mapq0_frac: float = 0.0
    clip_frac: float = 0.01
    dup_frac: float = 0.002
    secondary_frac: float = 0.001
    improper_frac: float = 0.002
    noqual_frac: float = 0.0005
    repeat_frac: float = 0.0     # fraction of the reference in 2-20 kb repeat copies
    repeat_mapq_max: int = -1    # reads touching a repeat get mapq 0..max (-1: off)


def workload(cfg, scale=1.0):
    """The five workloads; `scale` < 1 shrinks genome sizes for quick tests."""
    if cfg == 1:
        return Workload("small-50kb", 1001, [int(50_000 * scale)], gc=0.5, coverage=50, insert_mean=400,
                        insert_sd=50, n_snps=20, n_indels=5, indel_len=(1, 10), sub_err=0.005)
    if cfg == 2:
        return Workload("bacterial-5Mb-100x", 1002, [int(5_000_000 * scale)], gc=0.65, coverage=100,
                        insert_mean=500, insert_sd=80, n_snps=int(500 * scale) or 1, n_indels=int(100 * scale) or 1,
                        indel_len=(1, 30), sub_err=0.003, indel_err=0.0002, mapq0_frac=0.03)
    if cfg == 3:
        rng = np.random.Generator(np.random.PCG64(1003))
        n = max(1, int(round(3000 * scale)))
        # log-normal, median 20 kb; sigma 1.354 puts the mean near 50 kb (3,000 contigs ~ 150 Mb)
        lens = np.clip(np.exp(rng.normal(np.log(20_000), 1.354, size=n)), 1_000, 2_000_000).astype(np.int64)
        return Workload("draft-3000-contigs-40x", 1003, [int(x) for x in lens], gc=0.5, coverage=40,
                        insert_mean=400, insert_sd=50, variant_frac=0.01, indel_len=(1, 10), sub_err=0.003,
                        indel_err=0.0002)
    if cfg == 4:
        return Workload("eukaryotic-120Mb-repeats", 1004, [int(120_000_000 * scale)], gc=0.45, coverage=40,
                        insert_mean=400, insert_sd=50, n_snps=0, n_indels=int(2000 * scale) or 1,
                        indel_len=(10, 200), sub_err=0.003, indel_err=0.0002, repeat_frac=0.10,
                        repeat_mapq_max=3)
    raise ValueError(cfg)


def random_reference(rng, length, gc):
    p = [(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2]
    return np.frombuffer(b"ACGT", np.uint8)[rng.choice(4, size=length, p=p)]


def add_repeats(rng, ref, frac):
    """Copies 2-20 kb segments of the reference over other places until `frac`
    of it lies in repeat copies; returns the mask of copied bases."""
    mask = np.zeros(ref.size, np.uint8)
    target = int(frac * ref.size)
    done = 0
    while done < target and ref.size > 50_000:
        ln = int(rng.integers(2_000, 20_001))
        src = int(rng.integers(0, ref.size - ln))
        dst = int(rng.integers(0, ref.size - ln))
        if abs(src - dst) < ln:
            continue
        ref[dst:dst + ln] = ref[src:src + ln]
        mask[dst:dst + ln] = 1
        mask[src:src + ln] = 1
        done += ln
    return mask


def plant_variants(rng, ref, n_snps, n_indels, indel_len):
    """Plants SNPs and indels (>= 300 bp apart, away from the ends) in a copy
    of `ref`.  Returns (sample, sample_to_ref, variants) where variants are
    (ref_pos_1based, kind, ref_allele, alt_allele)."""
    L = ref.size
    n = n_snps + n_indels
    if n == 0 or L < 2000:
        return ref.copy(), np.arange(L, dtype=np.int64), []
    slots = max(1, (L - 1000) // 300)
    n = min(n, slots)
    pick = np.sort(rng.choice(slots, size=n, replace=False))
    positions = 500 + pick * 300 + rng.integers(0, 100, size=n)
    kinds = np.array(["snp"] * min(n_snps, n) + ["ins", "del"] * n)[:n]
    rng.shuffle(kinds)
    pieces, maps, variants = [], [], []
    cur = 0
    acgt = np.frombuffer(b"ACGT", np.uint8)
    for p, k in zip(positions.tolist(), kinds.tolist()):
        if k == "snp":
            pieces.append(ref[cur:p]); maps.append(np.arange(cur, p))
            alt = acgt[(np.where(acgt == ref[p])[0][0] + 1 + rng.integers(0, 3)) % 4] if ref[p] in acgt else acgt[0]
            pieces.append(np.array([alt], np.uint8)); maps.append(np.array([p]))
            variants.append((p + 1, "snp", chr(ref[p]), chr(alt)))
            cur = p + 1
        elif k == "ins":
            ln = int(rng.integers(indel_len[0], indel_len[1] + 1))
            ins = acgt[rng.integers(0, 4, size=ln)]
            pieces.append(ref[cur:p + 1]); maps.append(np.arange(cur, p + 1))
            pieces.append(ins); maps.append(np.full(ln, -1))
            variants.append((p + 1, "ins", "", ins.tobytes().decode()))
            cur = p + 1
        else:
            ln = int(rng.integers(indel_len[0], indel_len[1] + 1))
            pieces.append(ref[cur:p + 1]); maps.append(np.arange(cur, p + 1))
            variants.append((p + 2, "del", ref[p + 1:p + 1 + ln].tobytes().decode(), ""))
            cur = p + 1 + ln
    pieces.append(ref[cur:]); maps.append(np.arange(cur, L))
    return (np.concatenate(pieces).astype(np.uint8), np.concatenate(maps).astype(np.int64), variants)


def simulate_contig(sample, s2r, ref_len, w, ref_id, seed, repeat_mask=None):
    lib = _lib()
    P = _SimParams(read_len=w.read_len, coverage=w.coverage, insert_mean=w.insert_mean, insert_sd=w.insert_sd,
                   sub_err=w.sub_err, indel_err=w.indel_err, n_frac=w.n_frac, mapq0_frac=w.mapq0_frac,
                   clip_frac=w.clip_frac, dup_frac=w.dup_frac, secondary_frac=w.secondary_frac,
                   improper_frac=w.improper_frac, noqual_frac=w.noqual_frac, ref_id=ref_id,
                   repeat_mapq_max=w.repeat_mapq_max)
    sample = np.ascontiguousarray(sample, np.uint8)
    s2r = np.ascontiguousarray(s2r, np.int64)
    rm = None if repeat_mask is None else np.ascontiguousarray(repeat_mask, np.uint8)
    h = lib.sy_simulate(sample.ctypes.data, sample.size, s2r.ctypes.data, rm.ctypes.data if rm is not None else None,
                        ref_len, C.byref(P), C.c_uint64(seed))
    try:
        n = lib.sy_n_reads(h)
        nc = lib.sy_n_cigar(h)
        L = w.read_len
        st = ReadStore(pos=np.empty(n, np.int32), aend=np.empty(n, np.int32), flag=np.empty(n, np.uint16),
                       mapq=np.empty(n, np.uint8), tlen=np.empty(n, np.int32), ref_id=np.empty(n, np.int32),
                       mate_ref_id=np.empty(n, np.int32), cigar_off=np.empty(n, np.int64),
                       n_cigar=np.empty(n, np.uint16), cigar=np.empty(nc, np.uint32), seq_off=np.empty(n, np.int64),
                       l_seq=np.empty(n, np.int32), seq=np.empty(n * ((L + 1) // 2), np.uint8),
                       qual_off=np.empty(n, np.int64), qual=np.empty(n * L, np.uint8))
        lib.sy_copy(h, st.pos.ctypes.data, st.aend.ctypes.data, st.flag.ctypes.data, st.mapq.ctypes.data,
                    st.tlen.ctypes.data, st.ref_id.ctypes.data, st.cigar_off.ctypes.data, st.n_cigar.ctypes.data,
                    st.cigar.ctypes.data, st.seq_off.ctypes.data, st.l_seq.ctypes.data, st.seq.ctypes.data,
                    st.qual_off.ctypes.data, st.qual.ctypes.data)
        st.mate_ref_id[:] = st.ref_id
        st.name_id = np.empty(n, np.int64)
        lib.sy_copy_pairs(h, st.name_id.ctypes.data)
    finally:
        lib.sy_free(h)
    return st


@dataclass
class Dataset:
    workload: Workload
    names: list
    contigs: list          # uint8 ASCII arrays (the reference)
    reads: ReadStore       # sorted by (ref_id, pos)
    variants: list         # per contig


def generate(cfg_or_workload, scale=1.0, threads=None):
    """The workload's reference, planted variants and coordinate-sorted reads.
    Contigs are simulated concurrently; every contig has its own seed, so the
    result does not depend on the thread count."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    w = workload(cfg_or_workload, scale) if isinstance(cfg_or_workload, int) else cfg_or_workload
    rng = np.random.Generator(np.random.PCG64(w.seed))
    total = sum(w.contig_lengths)
    names, contigs, jobs, variants = [], [], [], []
    for ci, ln in enumerate(w.contig_lengths):
        ref = random_reference(rng, ln, w.gc)
        rmask = add_repeats(rng, ref, w.repeat_frac) if w.repeat_frac > 0 else None
        if w.variant_frac > 0:
            nv = max(1, int(w.variant_frac * ln))
            ns, ni = int(nv * 0.8), nv - int(nv * 0.8)
            # 1% of bases carry variants: pack them densely (every ~100 bp)
            sample, s2r, var = _plant_dense(rng, ref, ns, ni, w.indel_len)
        else:
            ns = int(round(w.n_snps * ln / total))
            ni = int(round(w.n_indels * ln / total))
            sample, s2r, var = plant_variants(rng, ref, ns, ni, w.indel_len)
        seed = int(rng.integers(0, 2**63 - 1))
        jobs.append((sample, s2r, ln, ci, seed, rmask))
        names.append(f"contig{ci + 1}" if len(w.contig_lengths) > 1 else "chr1")
        contigs.append(ref)
        variants.append(var)
    nt = threads or min(len(jobs), os.cpu_count() or 1)
    if nt > 1 and len(jobs) > 1:
        with ThreadPoolExecutor(nt) as ex:
            stores = list(ex.map(lambda j: simulate_contig(j[0], j[1], j[2], w, j[3], j[4], j[5]), jobs))
    else:
        stores = [simulate_contig(j[0], j[1], j[2], w, j[3], j[4], j[5]) for j in jobs]
    reads = stores[0] if len(stores) == 1 else concat_stores(stores)
    return Dataset(w, names, contigs, reads, variants)


def _plant_dense(rng, ref, n_snps, n_indels, indel_len):
    L = ref.size
    n = n_snps + n_indels
    if L < 2000 or n == 0:
        return ref.copy(), np.arange(L, dtype=np.int64), []
    spacing = max(30, (L - 1000) // max(n, 1))
    slots = max(1, (L - 1000) // spacing)
    n = min(n, slots)
    pos = 500 + np.arange(n) * spacing + rng.integers(0, max(1, spacing - 20), size=n)
    kinds = np.array(["snp"] * min(n_snps, n) + ["ins", "del"] * n)[:n]
    rng.shuffle(kinds)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    pieces, maps, variants = [], [], []
    cur = 0
    for p, k in zip(pos.tolist(), kinds.tolist()):
        if p < cur + 1:
            continue
        if k == "snp":
            pieces.append(ref[cur:p]); maps.append(np.arange(cur, p))
            alt = acgt[(np.where(acgt == ref[p])[0][0] + 1 + rng.integers(0, 3)) % 4]
            pieces.append(np.array([alt], np.uint8)); maps.append(np.array([p]))
            variants.append((p + 1, "snp", chr(ref[p]), chr(alt)))
            cur = p + 1
        elif k == "ins":
            ln = int(rng.integers(indel_len[0], indel_len[1] + 1))
            ins = acgt[rng.integers(0, 4, size=ln)]
            pieces.append(ref[cur:p + 1]); maps.append(np.arange(cur, p + 1))
            pieces.append(ins); maps.append(np.full(ln, -1))
            variants.append((p + 1, "ins", "", ins.tobytes().decode()))
            cur = p + 1
        else:
            ln = int(rng.integers(indel_len[0], min(indel_len[1], spacing // 3) + 1))
            pieces.append(ref[cur:p + 1]); maps.append(np.arange(cur, p + 1))
            variants.append((p + 2, "del", ref[p + 1:p + 1 + ln].tobytes().decode(), ""))
            cur = p + 1 + ln
    pieces.append(ref[cur:]); maps.append(np.arange(cur, L))
    return (np.concatenate(pieces).astype(np.uint8), np.concatenate(maps).astype(np.int64), variants)
