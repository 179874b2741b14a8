"""pg_phys_cov_scan_static: the physical-coverage scan for callers that cannot
let the library allocate device memory (their own pool already holds it).

The entry point is called through the C ABI on caller-owned device buffers
and must reproduce, bit for bit, the physical coverage and insert size that
the regular entry point (pg_pileup_regions) computes for the same regions.
It is called several times in a row on regions of different sizes, because
every call reuses the library's one static scratch array.  This file sorts
last so that a failure here does not stop the other GPU tests.
"""
import ctypes as C

import numpy as np
import pytest

from pilon_gb300 import _abi, synth

pytestmark = pytest.mark.gpu


def _diff_arrays(ds, params, region):
    """physCovIncr (S/PileUpRegion.scala:62-88) over the reads fed to the region:
    the +1/-1 and +size/-size difference arrays and the carry from reads that
    start before the region."""
    c, s, e, rb, re = region
    R = ds.reads
    n = e - s + 1
    pos = R.pos[rb:re].astype(np.int64)
    aend = R.aend[rb:re].astype(np.int64)
    fl = R.flag[rb:re].astype(np.int64)
    tlen = R.tlen[rb:re].astype(np.int64)
    clen = ds.contigs[c].size
    qs, qe = max(s - 10000, 0), min(e + 10000, clen)
    end = np.where(fl & 4, pos, aend)
    fed = (R.ref_id[rb:re] == c) & (pos <= qe) & (end >= qs)
    fed &= ((fl & 0x200) == 0) & ((fl & 0x400) == 0) & ((fl & 0x100) == 0)
    paired = (fl & 1) != 0
    valid = (R.mapq[rb:re] >= params.min_mq) & (~paired | (((fl & 2) != 0) &
                                                          (R.ref_id[rb:re] == R.mate_ref_id[rb:re])))
    use = fed & valid & ~(paired & (tlen <= 0))
    st = np.where(~paired, np.minimum(pos, aend), np.where(tlen > 0, pos, aend + 1 + tlen))
    en = np.where(~paired, np.maximum(pos, aend), np.where(tlen > 0, pos + tlen, aend + 1))
    size = en - st
    pd = np.zeros(n, np.int64)
    idf = np.zeros(n, np.int64)
    a = use & (st >= s) & (st <= e)
    np.add.at(pd, st[a] - s, 1)
    np.add.at(idf, st[a] - s, size[a])
    carry = use & (st < s) & (en >= s)
    b = use & (en >= s) & (en <= e)
    np.add.at(pd, en[b] - s, -1)
    np.add.at(idf, en[b] - s, -size[b])
    wrap = lambda x: ((x + 2**31) % 2**32 - 2**31).astype(np.int32)
    return wrap(pd), wrap(idf), int(carry.sum()), int(size[carry].sum())


def test_static_scan_matches_pileup_regions():
    import torch
    from pilon_gb300.engine import Engine, lib
    from pilon_gb300.regions import plan_regions

    ds = synth.generate(1)
    params = _abi.default_params()
    regions = plan_regions(ds.reads, [c.size for c in ds.contigs], chunk_size=17_000)
    assert len(regions) >= 3
    eng = Engine(0)
    try:
        eng.set_reference(ds.contigs)
        eng.set_reads(ds.reads)
        eng.pileup_regions(regions, params)
        expected = [eng.fetch(r) for r in range(len(regions))]
    finally:
        eng.close()

    L = lib()
    f = L.pg_phys_cov_scan_static
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_char_p, C.c_int32]
    err = C.create_string_buffer(256)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    # several calls in a row, regions of different sizes, then the first again
    for r in [0, 1, 2, 0]:
        pd, idf, carry_pc, carry_is = _diff_arrays(ds, params, regions[r])
        ex = expected[r]
        assert carry_pc == ex.stats.phys_cov_start and carry_is == ex.stats.insert_size_start
        d_pd = torch.from_numpy(pd).to(dev)
        d_id = torch.from_numpy(idf).to(dev)
        d_pc = torch.full_like(d_pd, -7)
        d_is = torch.full_like(d_id, -7)
        torch.cuda.synchronize(dev)
        rc = f(d_pd.data_ptr(), d_id.data_ptr(), pd.size, carry_pc, carry_is, d_pc.data_ptr(), d_is.data_ptr(),
               C.c_void_p(stream.cuda_stream), err, 256)
        assert rc == _abi.PG_OK, err.value.decode()
        torch.cuda.synchronize(dev)
        assert np.array_equal(d_pc.cpu().numpy(), ex.phys_cov), f"region {r}: physical coverage differs"
        assert np.array_equal(d_is.cpu().numpy(), ex.insert_size), f"region {r}: insert size differs"


def _scan_fn():
    from pilon_gb300.engine import lib
    f = lib().pg_phys_cov_scan_static
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_char_p, C.c_int32]
    return f


def _expected_scan(pd, idf, carry_pc, carry_is):
    """computePhysCov (S/PileUpRegion.scala:90-100) in numpy: Int prefix sums
    that wrap at 32 bits, then insertSize / physCov (truncating) where
    physCov > 0."""
    wrap = lambda x: ((x + 2**31) % 2**32 - 2**31)
    pc = wrap(np.cumsum(pd.astype(np.int64)) + carry_pc)
    isz = wrap(np.cumsum(idf.astype(np.int64)) + carry_is)
    q = np.sign(isz) * (np.abs(isz) // np.where(pc > 0, pc, 1))
    return pc.astype(np.int32), np.where(pc > 0, q, isz).astype(np.int32)


@pytest.mark.parametrize("n", [3_000_017, _abi.PG_STATIC_SCAN_MAX_POSITIONS])
def test_static_scan_long_regions_and_in_place(n):
    """Regions above 1,048,576 positions take the tile scan over several rounds
    of 1024 tiles, up to the size limit; output written over the input gives the
    same values.  Random difference arrays, small and full-range (wrapping)."""
    import torch
    f = _scan_fn()
    err = C.create_string_buffer(256)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(n)
    cases = [(rng.integers(-3, 4, n).astype(np.int32), rng.integers(-900, 901, n).astype(np.int32), 7, 3500),
             (rng.integers(-2**31, 2**31, n, dtype=np.int64).astype(np.int32),
              rng.integers(-2**31, 2**31, n, dtype=np.int64).astype(np.int32), -5, 2**31 - 9)]
    for pd, idf, c_pc, c_is in cases:
        want_pc, want_is = _expected_scan(pd, idf, c_pc, c_is)
        d_pd = torch.from_numpy(pd).to(dev)
        d_id = torch.from_numpy(idf).to(dev)
        d_pc = torch.full_like(d_pd, -7)
        d_is = torch.full_like(d_id, -7)
        torch.cuda.synchronize(dev)
        rc = f(d_pd.data_ptr(), d_id.data_ptr(), n, c_pc, c_is, d_pc.data_ptr(), d_is.data_ptr(),
               C.c_void_p(stream.cuda_stream), err, 256)
        assert rc == _abi.PG_OK, err.value.decode()
        # in place: the output arrays are the input arrays
        rc = f(d_pd.data_ptr(), d_id.data_ptr(), n, c_pc, c_is, d_pd.data_ptr(), d_id.data_ptr(),
               C.c_void_p(stream.cuda_stream), err, 256)
        assert rc == _abi.PG_OK, err.value.decode()
        torch.cuda.synchronize(dev)
        assert np.array_equal(d_pc.cpu().numpy(), want_pc)
        assert np.array_equal(d_is.cpu().numpy(), want_is)
        assert np.array_equal(d_pd.cpu().numpy(), want_pc), "in place"
        assert np.array_equal(d_id.cpu().numpy(), want_is), "in place"
        del d_pd, d_id, d_pc, d_is


def test_static_scan_rejects_oversize():
    f = _scan_fn()
    err = C.create_string_buffer(256)
    one = np.zeros(1, np.int32)
    p = one.ctypes.data  # never dereferenced: the size check comes first
    rc = f(p, p, _abi.PG_STATIC_SCAN_MAX_POSITIONS + 1, 0, 0, p, p, None, err, 256)
    assert rc == _abi.PG_ERR_LIMIT
    assert b"exceed" in err.value
