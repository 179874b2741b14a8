// pg_pileup.cu — pileup construction kernels.
//
//   k_read_extent   maxima of how far a read's walk reaches around its start
//   k_tile_ranges   per walk tile: the range of (position-sorted) reads that can touch it
//   k_walk          the CIGAR walk of PileUpRegion.addRead for M/=/X and S operators
//                   (S/PileUpRegion.scala:145-216): one CTA owns a tile of positions,
//                   accumulates PileUp.add / badPair / clips with shared-memory
//                   integer atomics and writes the tile's records once
//   k_read_events   per (region, read): BamFile.process bookkeeping (readCount,
//                   addInsert), physCovIncr, and the I/D operators with their left
//                   shift (S/PileUpRegion.scala:150-183), applied with global atomics
//                   after k_walk and logged as events for the indel vote
//   k_event_scatter events -> per-call-tile buckets
//   k_scan_*        computePhysCov (S/PileUpRegion.scala:90-100) as a segmented scan
#include <cuda_runtime.h>

#include <algorithm>

#include "pg_internal.cuh"

namespace pg {

#define FULL 0xffffffffu

__device__ inline bool consumes_read(int op) { return op == 0 || op == 1 || op == 4 || op == 7 || op == 8; }
__device__ inline bool consumes_ref(int op) { return op == 0 || op == 2 || op == 3 || op == 7 || op == 8; }

// validateRead (S/BamFile.scala:101-105)
__device__ inline bool validate_read(uint16_t fl, const DevParams& P) {
  return (P.nonpf || !(fl & 0x200)) && (P.duplicates || !(fl & 0x400)) && !(fl & 0x100);
}

// queryOverlapping(name, qs, qe) keeps reads whose [start, end] overlaps the
// window; an unmapped read placed at a position counts as [pos, pos].
__device__ inline bool in_window(int32_t pos, int32_t aend, uint16_t fl, const RegionDev& g) {
  int32_t e = (fl & 0x4) ? pos : aend;
  return pos <= g.qe && e >= g.qs;
}

// ---------------------------------------------------------------------------
// Also validates the store: every read's CIGAR, bases and qualities must lie
// inside their arrays, and positions must not decrease within a reference.
__global__ void k_read_extent(Reads R, ReadExtent* out) {
  int32_t lead = 0, back = 0;
  unsigned long long nid = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < R.n; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t pos = R.pos[i];
    {
      const int64_t co0 = R.cigar_off[i], so0 = R.seq_off[i], qo0 = R.qual_off[i];
      const int32_t L = R.l_seq[i];
      const bool bad = co0 < 0 || co0 + R.n_cigar[i] > R.n_cigar_words || L < 0 || so0 < 0 ||
                       so0 + (L + 1) / 2 > R.seq_bytes || qo0 < 0 || qo0 + L > R.qual_bytes;
      if (bad) {
        atomicCAS(&out->bad_read, 0ull, (unsigned long long)i + 1);
        continue;
      }
      if (i > 0 && R.ref_id[i] == R.ref_id[i - 1] && pos < R.pos[i - 1]) out->unsorted = 1;
    }
    int64_t lo = pos, hi = pos;
    int32_t ro = 0, fo = 0;
    int64_t co = R.cigar_off[i];
    int nc = R.n_cigar[i];
    for (int k = 0; k < nc; k++) {
      uint32_t w = R.cigar[co + k];
      int32_t len = (int32_t)(w >> 4);
      int op = (int)(w & 15);
      int64_t locus = (int64_t)pos + fo;
      if (op == 0 || op == 7 || op == 8) {
        if (len > 0) { lo = min(lo, locus); hi = max(hi, locus + len - 1); }
      } else if (op == 4) {
        int64_t cs = ro == 0 ? locus - len : locus;
        if (len > 0) { lo = min(lo, cs); hi = max(hi, cs + len - 1); }
      } else if (op == 1 || op == 2) {
        nid++;
      }
      if (consumes_read(op)) ro += len;
      if (consumes_ref(op)) fo += len;
    }
    lead = max(lead, (int32_t)min((long long)(pos - lo), (long long)(1 << 30)));
    back = max(back, (int32_t)min((long long)(hi - pos), (long long)(1 << 30)));
  }
  lead = __reduce_max_sync(FULL, lead);
  back = __reduce_max_sync(FULL, back);
  for (int o = 16; o > 0; o >>= 1) nid += __shfl_down_sync(FULL, nid, o);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out->max_lead, lead);
    atomicMax(&out->max_back, back);
    atomicAdd(&out->n_indel_ops, nid);
  }
}

void launch_read_extent(const Reads& R, ReadExtent* out, cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(ReadExtent), s);
  if (R.n == 0) return;
  int blocks = (int)std::min<int64_t>((R.n + 255) / 256, 152 * 16);
  k_read_extent<<<blocks, 256, 0, s>>>(R, out);
}

// ---------------------------------------------------------------------------
__device__ inline int64_t lower_bound_pos(const int32_t* pos, int64_t lo, int64_t hi, int64_t v) {
  while (lo < hi) {
    int64_t m = (lo + hi) >> 1;
    if ((int64_t)pos[m] < v) lo = m + 1; else hi = m;
  }
  return lo;
}

__global__ void k_tile_ranges(Reads R, const RegionDev* regions, WalkTile* tiles, int32_t n_tiles,
                              const ReadExtent* ext) {
  int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tiles) return;
  WalkTile& T = tiles[t];
  const RegionDev& g = regions[T.region];
  int64_t tlo = (int64_t)g.start + T.lo, thi = tlo + T.len - 1;
  int64_t a = tlo - ext->max_back, b = thi + ext->max_lead + 1;
  T.read_lo = lower_bound_pos(R.pos, g.read_begin, g.read_end, a);
  T.read_hi = lower_bound_pos(R.pos, T.read_lo, g.read_end, b);
}

void launch_tile_ranges(const Reads& R, const RegionDev* regions, WalkTile* tiles, int32_t n_tiles,
                        const ReadExtent* ext, cudaStream_t s) {
  if (n_tiles == 0) return;
  k_tile_ranges<<<(n_tiles + 255) / 256, 256, 0, s>>>(R, regions, tiles, n_tiles, ext);
}

// ---------------------------------------------------------------------------
// The walk kernel.  Shared memory holds 12 uint32 counters per tile position:
//   cnt[4] | qs[4] | mq | q | bad | clips          (each an array of tile_width)
// qs fits uint32 exactly while a pass adds at most kMaxReadsPerPass reads of
// qual <= 127 and mq <= 255 to one position; tiles with more reads run in
// several passes and add each pass's sums into the records.
__global__ void __launch_bounds__(512) k_walk(WalkArgs a, int32_t tile_begin, int32_t tile_end) {
  extern __shared__ uint32_t sm[];
  const int T = a.tile_width;
  uint32_t* s_cnt = sm;
  uint32_t* s_qs = sm + 4 * T;
  uint32_t* s_mq = sm + 8 * T;
  uint32_t* s_q = sm + 9 * T;
  uint32_t* s_bad = sm + 10 * T;
  uint32_t* s_clip = sm + 11 * T;
  __shared__ unsigned long long s_bc;

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const Reads& R = a.R;
  const DevParams& P = a.P;

  for (int32_t t = tile_begin + blockIdx.x; t < tile_end; t += gridDim.x) {
    const WalkTile tile = a.tiles[t];
    const RegionDev g = a.regions[tile.region];
    const int32_t tileLo = g.start + tile.lo, tileHi = tileLo + tile.len - 1;
    const uint8_t* cref = a.ref + g.ref_off;
    unsigned long long bc = 0;
    if (threadIdx.x == 0) s_bc = 0;

    for (int64_t c0 = tile.read_lo, pass = 0; pass == 0 || c0 < tile.read_hi; c0 += kMaxReadsPerPass, pass++) {
      const int64_t c1 = min(c0 + kMaxReadsPerPass, tile.read_hi);
      for (int k = threadIdx.x; k < 12 * T; k += blockDim.x) sm[k] = 0;
      __syncthreads();

      for (int64_t base = c0 + (int64_t)warp * 32; base < c1; base += (int64_t)nwarps * 32) {
        const int64_t i = base + lane;
        bool ok = i < c1;
        int32_t h_pos = 0, h_aend = 0, h_len = 0, h_nc = 0, h_tlen = 0;
        uint16_t h_flag = 0;
        uint8_t h_mq = 0;
        int64_t h_co = 0, h_qo = 0;
        if (ok) {
          h_pos = R.pos[i]; h_aend = R.aend[i]; h_flag = R.flag[i];
          ok = R.ref_id[i] == g.contig && in_window(h_pos, h_aend, h_flag, g) && validate_read(h_flag, P);
        }
        if (ok) {
          h_len = R.l_seq[i]; h_nc = R.n_cigar[i]; h_mq = R.mapq[i]; h_co = R.cigar_off[i]; h_qo = R.qual_off[i];
          const bool paired = h_flag & 0x1;
          const bool valid = (h_mq >= P.min_mq) &&
                             (!paired || ((h_flag & 0x2) && R.ref_id[i] == R.mate_ref_id[i]));
          h_tlen = valid ? 1 : 0;  // reuse as the `valid` bit
        }
        unsigned todo = __ballot_sync(FULL, ok);
        while (todo) {
          const int src = __ffs(todo) - 1;
          todo &= todo - 1;
          const int64_t ri = base + src;
          const int32_t pos = __shfl_sync(FULL, h_pos, src);
          const int32_t length = __shfl_sync(FULL, h_len, src);
          const int32_t nc = __shfl_sync(FULL, h_nc, src);
          const int32_t mq = (int32_t)__shfl_sync(FULL, (int32_t)h_mq, src);
          const bool valid = __shfl_sync(FULL, h_tlen, src) != 0;
          const int64_t co = __shfl_sync(FULL, h_co, src);
          const int64_t qo = __shfl_sync(FULL, h_qo, src);
          const int64_t so = R.seq_off[ri];

          // clipped bases -> adjusted mapping quality (S/PileUpRegion.scala:139-141)
          int32_t clipped = 0;
          for (int cb = 0; cb < nc; cb += 32) {
            uint32_t w = (cb + lane < nc) ? R.cigar[co + cb + lane] : 0u;
            int32_t sl = ((w & 15u) == 4u) ? (int32_t)(w >> 4) : 0;
            clipped += __reduce_add_sync(FULL, sl);
          }
          const int32_t adjMq = roundDivI(wmul(mq, length - clipped), length);
          const uint32_t mq1 = (uint32_t)(adjMq + 1);
          const bool hasQual = length > 0 && R.qual[qo] != 0xFF;

          int32_t readOffset = 0, refOffset = 0;
          for (int cb = 0; cb < nc; cb += 32) {
            uint32_t wl = (cb + lane < nc) ? R.cigar[co + cb + lane] : 0u;
            const int kmax = min(32, nc - cb);
            for (int k = 0; k < kmax; k++) {
              const uint32_t w = __shfl_sync(FULL, wl, k);
              const int32_t len = (int32_t)(w >> 4);
              const int op = (int)(w & 15u);
              const int32_t locus = pos + refOffset;
              if (op == 0 || op == 7 || op == 8) {
                int32_t i0 = max(max(tileLo - locus, P.flank - readOffset), 0);
                int32_t i1 = min(min(tileHi - locus + 1, length - P.flank - readOffset), len);
                for (int32_t ii = i0 + lane; ii < i1; ii += 32) {
                  const int32_t rOff = readOffset + ii;
                  const int32_t p = locus + ii - tileLo;
                  int32_t qual = hasQual ? (int32_t)(int8_t)R.qual[qo + rOff] : P.default_qual;
                  if (P.long_read == PG_NANOPORE) {  // nanoporeExclude(index(locusPlus)), contig-indexed
                    const int32_t i0x = locus + ii - g.start;
                    if (i0x - 2 >= 0 && i0x + 2 <= g.size - 1 && cref[i0x - 2] == 'C' && cref[i0x - 1] == 'C' &&
                        cref[i0x + 1] == 'G' && cref[i0x + 2] == 'G')
                      qual = 0;
                  }
                  if (valid) {
                    const uint8_t byte = R.seq[so + (rOff >> 1)];
                    const uint32_t nib = (rOff & 1) ? (byte & 15u) : (uint32_t)(byte >> 4);
                    const int bi = nib_index(nib);
                    if (bi >= 0 && qual >= P.min_qual) {
                      atomicAdd(&s_cnt[bi * T + p], 1u);
                      atomicAdd(&s_qs[bi * T + p], (uint32_t)qual * mq1);
                      atomicAdd(&s_mq[p], mq1);
                      atomicAdd(&s_q[p], (uint32_t)qual);
                    }
                    bc++;
                  } else {
                    atomicAdd(&s_bad[p], 1u);
                  }
                }
              } else if (op == 4) {
                const int32_t clipStart = readOffset == 0 ? locus - len : locus;
                const int32_t clipEnd = clipStart + len - 1;
                if (lane == 0) {
                  if (clipStart >= tileLo && clipStart <= tileHi) atomicAdd(&s_clip[clipStart - tileLo], 1u);
                  if (clipEnd >= tileLo && clipEnd <= tileHi) atomicAdd(&s_clip[clipEnd - tileLo], 1u);
                }
                int32_t i0 = max(tileLo - clipStart, 0);
                int32_t i1 = min(tileHi - clipStart + 1, len);
                for (int32_t ii = i0 + lane; ii < i1; ii += 32) atomicAdd(&s_bad[clipStart + ii - tileLo], 1u);
              }
              if (op == 0 || op == 1 || op == 4 || op == 7 || op == 8) readOffset += len;
              if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) refOffset += len;
            }
          }
        }
      }
      __syncthreads();

      // flush: the first pass stores, later passes add (the CTA owns the tile)
      for (int32_t p = threadIdx.x; p < tile.len; p += blockDim.x) {
        const int64_t gp = g.pos_base + tile.lo + p;
        int4 c = make_int4((int)s_cnt[p], (int)s_cnt[T + p], (int)s_cnt[2 * T + p], (int)s_cnt[3 * T + p]);
        longlong2 q01 = make_longlong2((long long)s_qs[p], (long long)s_qs[T + p]);
        longlong2 q23 = make_longlong2((long long)s_qs[2 * T + p], (long long)s_qs[3 * T + p]);
        if (pass == 0) {
          a.rec.count[gp] = c;
          a.rec.qual_sum[2 * gp] = q01;
          a.rec.qual_sum[2 * gp + 1] = q23;
          a.rec.mq_sum[gp] = (int32_t)s_mq[p];
          a.rec.q_sum[gp] = (int32_t)s_q[p];
          a.rec.bad_pair[gp] = (int32_t)s_bad[p];
          a.rec.clips[gp] = (int32_t)s_clip[p];
          a.rec.deletions[gp] = 0;
          a.rec.del_qual[gp] = 0;
          a.rec.insertions[gp] = 0;
          a.rec.ins_qual[gp] = 0;
          a.rec.phys_cov[gp] = 0;
          a.rec.insert_size[gp] = 0;
        } else {
          int4 o = a.rec.count[gp];
          a.rec.count[gp] = make_int4(o.x + c.x, o.y + c.y, o.z + c.z, o.w + c.w);
          longlong2 o1 = a.rec.qual_sum[2 * gp], o2 = a.rec.qual_sum[2 * gp + 1];
          a.rec.qual_sum[2 * gp] = make_longlong2(o1.x + q01.x, o1.y + q01.y);
          a.rec.qual_sum[2 * gp + 1] = make_longlong2(o2.x + q23.x, o2.y + q23.y);
          a.rec.mq_sum[gp] = wadd(a.rec.mq_sum[gp], (int32_t)s_mq[p]);
          a.rec.q_sum[gp] = wadd(a.rec.q_sum[gp], (int32_t)s_q[p]);
          a.rec.bad_pair[gp] = wadd(a.rec.bad_pair[gp], (int32_t)s_bad[p]);
          a.rec.clips[gp] = wadd(a.rec.clips[gp], (int32_t)s_clip[p]);
        }
      }
      __syncthreads();
    }
    // region baseCount (PileUpRegion.add counts every in-region base of a valid read)
    for (int o = 16; o > 0; o >>= 1) bc += __shfl_down_sync(FULL, bc, o);
    if (lane == 0 && bc) atomicAdd(&s_bc, bc);
    __syncthreads();
    if (threadIdx.x == 0 && s_bc) atomicAdd(&a.stats[tile.region].base_count, s_bc);
    __syncthreads();
  }
}

void launch_walk(const WalkArgs& a, int32_t tile_begin, int32_t tile_count, int warps, cudaStream_t s) {
  if (tile_count <= 0) return;
  size_t smem = (size_t)12 * a.tile_width * sizeof(uint32_t);
  static size_t configured = 0;
  if (smem > configured) {
    cudaFuncSetAttribute(k_walk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = smem;
  }
  int per_sm = max(1, (int)((227 * 1024) / (smem + 1024)));
  int blocks = min(tile_count, 152 * per_sm);
  k_walk<<<blocks, warps * 32, smem, s>>>(a, tile_begin, tile_begin + tile_count);
}

// ---------------------------------------------------------------------------
// Per (region, read): readCount, insert statistics, physCovIncr and indels.
__device__ inline int32_t read_qual(const Reads& R, int64_t i, int32_t k, bool hasQual, const DevParams& P) {
  return hasQual ? (int32_t)(int8_t)R.qual[R.qual_off[i] + k] : P.default_qual;
}

__global__ void __launch_bounds__(256) k_read_events(EventArgs a, int32_t chunk_begin, int32_t chunk_end) {
  __shared__ unsigned long long s_rc, s_bc, s_frc, s_frs, s_frq, s_rfc, s_rfs, s_rfq;
  __shared__ int32_t s_pcs, s_iss, s_err;
  const Reads& R = a.R;
  const DevParams& P = a.P;
  for (int32_t ch = chunk_begin + blockIdx.x; ch < chunk_end; ch += gridDim.x) {
    const ReadChunk C = a.chunks[ch];
    const RegionDev g = a.regions[C.region];
    const uint8_t* cref = a.ref + g.ref_off;
    if (threadIdx.x == 0) {
      s_rc = s_bc = s_frc = s_frs = s_frq = s_rfc = s_rfs = s_rfq = 0;
      s_pcs = s_iss = s_err = 0;
    }
    __syncthreads();
    auto inRegion = [&](int64_t l) { return l >= g.start && l <= g.stop; };
    for (int64_t i = C.lo + threadIdx.x; i < C.hi; i += blockDim.x) {
      const int32_t pos = R.pos[i], aend = R.aend[i];
      const uint16_t fl = R.flag[i];
      if (R.ref_id[i] != g.contig || !in_window(pos, aend, fl, g) || !validate_read(fl, P)) continue;
      atomicAdd(&s_rc, 1ull);
      const int32_t length = R.l_seq[i];
      const int32_t mq = R.mapq[i];
      const bool paired = fl & 0x1;
      const bool valid = (mq >= P.min_mq) && (!paired || ((fl & 0x2) && R.ref_id[i] == R.mate_ref_id[i]));
      const int32_t tlen = R.tlen[i];

      // physCovIncr (S/PileUpRegion.scala:62-88) and addInsert (S/BamFile.scala:194-202)
      int32_t insertSize = 0;
      if (valid && !(paired && tlen <= 0)) {
        int32_t s, e;
        if (!paired) { s = min(pos, aend); e = max(pos, aend); }
        else if (tlen > 0) { s = pos; e = wadd(pos, tlen); }
        else { s = wadd(wadd(aend, 1), tlen); e = aend + 1; }
        insertSize = wsub(e, s);
        if (inRegion(s)) {
          int64_t gp = g.pos_base + (s - g.start);
          atomicAdd(&a.rec.phys_cov[gp], 1);
          atomicAdd(&a.rec.insert_size[gp], insertSize);
        } else if (s < g.start && !(e < g.start)) {
          atomicAdd(&s_pcs, 1);
          atomicAdd(&s_iss, insertSize);
        }
        if (inRegion(e)) {
          int64_t gp = g.pos_base + (e - g.start);
          atomicAdd(&a.rec.phys_cov[gp], -1);
          atomicAdd(&a.rec.insert_size[gp], -insertSize);
        }
      }
      if (insertSize > 0 && insertSize < P.huge) {
        const bool rc = fl & 0x10;
        const bool fr = (insertSize > 0) ^ rc;
        const unsigned long long sq = (unsigned long long)(long long)wmul(insertSize, insertSize);
        if (fr) { atomicAdd(&s_frc, 1ull); atomicAdd(&s_frs, (unsigned long long)insertSize); atomicAdd(&s_frq, sq); }
        else { atomicAdd(&s_rfc, 1ull); atomicAdd(&s_rfs, (unsigned long long)insertSize); atomicAdd(&s_rfq, sq); }
      }

      // I and D operators (S/PileUpRegion.scala:150-183)
      const int64_t co = R.cigar_off[i];
      const int nc = R.n_cigar[i];
      bool anyIndel = false;
      int32_t clipped = 0;
      for (int k = 0; k < nc; k++) {
        uint32_t w = R.cigar[co + k];
        int op = (int)(w & 15u);
        if (op == 1 || op == 2) anyIndel = true;
        if (op == 4) clipped += (int32_t)(w >> 4);
      }
      if (!anyIndel || !valid) continue;
      const int32_t adjMq = roundDivI(wmul(mq, length - clipped), length);
      const int32_t indelMq = P.long_read > 0 ? min(adjMq, 8) : adjMq;
      const bool hasQual = length > 0 && R.qual[R.qual_off[i]] != 0xFF;
      auto trusted = [&](int32_t off) { return off >= P.flank && length - P.flank > off; };
      auto refAt = [&](int64_t k, bool& bad) -> uint8_t {
        if (k < 0 || k >= g.contig_len) { bad = true; return 0; }
        return cref[k];
      };
      auto homoRun = [&](int64_t i0, bool& bad) -> int64_t {  // PileUpRegion.addRead.homoRun (:120-126)
        uint8_t b0 = refAt(i0, bad);
        if (bad) return 0;
        for (int64_t k = i0 + 1; k < g.contig_len; k++)
          if (cref[k] != b0) return k - i0;
        return g.contig_len - i0;
      };
      int32_t readOffset = 0, refOffset = 0;
      for (int k = 0; k < nc; k++) {
        const uint32_t w = R.cigar[co + k];
        const int32_t len = (int32_t)(w >> 4);
        const int op = (int)(w & 15u);
        const int32_t locus = pos + refOffset;
        if (op == 1 && trusted(readOffset) && inRegion(locus)) {
          int32_t iloc = locus;
          int32_t rot = 0;
          bool bad = false;
          const int32_t avail = min(readOffset + len, length) - readOffset;
          while (iloc > 1) {
            uint8_t rb = refAt(iloc - 2, bad);
            if (bad) break;
            if (len - 1 < 0 || len - 1 >= avail) { bad = true; break; }
            int32_t kk = len - 1 - rot;  // last character of the rotated insertion
            if (kk < 0) kk += len;
            if (rb != nib_char(read_nib(R, i, readOffset + kk))) break;
            iloc -= 1;
            rot += 1;
            if (rot == len) rot = 0;
          }
          if (!bad && P.long_read > 0) {
            if (homoRun(iloc, bad) >= 4 && !bad) goto next_op;
          }
          if (bad || iloc < g.start) { atomicExch(&s_err, (int)PG_ERR_INDEX); goto next_op; }
          {
            const int64_t gp = g.pos_base + (iloc - g.start);
            atomicAdd(&a.rec.ins_qual[gp], indelMq + 1);
            atomicAdd(&a.rec.q_sum[gp], read_qual(R, i, readOffset, hasQual, P));
            atomicAdd(&a.rec.insertions[gp], 1);
            unsigned long long slot = atomicAdd(a.n_events, 1ull);
            if ((int64_t)slot < a.event_cap) {
              Event e;
              e.gpos = gp; e.read = i; e.region = C.region; e.len = len; e.roff = readOffset; e.kind_rot = rot;
              a.events[slot] = e;
            }
            atomicAdd(&a.bucket_count[g.call_tile0 + (iloc - g.start) / kCallTile], 1);
          }
        } else if (op == 2 && trusted(readOffset) && inRegion(locus) && inRegion((int64_t)locus + len - 1)) {
          int32_t dloc = locus, rloc = readOffset;
          bool bad = false;
          while (dloc > 1 && rloc > 0) {
            uint8_t x = refAt(dloc - 2, bad), y = refAt((int64_t)dloc + len - 2, bad);
            if (bad || x != y) break;
            dloc -= 1;
            rloc -= 1;
            if (trusted(rloc) && inRegion(dloc)) {
              if (inRegion((int64_t)dloc + len)) {  // add(dloc+len, base, qual, adjMq, valid = true)
                const int64_t gp = g.pos_base + (dloc + len - g.start);
                const int bi = nib_index(read_nib(R, i, rloc));
                const int32_t q = read_qual(R, i, rloc, hasQual, P);
                if (bi >= 0 && q >= P.min_qual) {
                  atomicAdd(((int*)a.rec.count) + 4 * gp + bi, 1);
                  atomicAdd(((unsigned long long*)a.rec.qual_sum) + 4 * gp + bi,
                            (unsigned long long)(long long)wmul(q, adjMq + 1));
                  atomicAdd(&a.rec.mq_sum[gp], adjMq + 1);
                  atomicAdd(&a.rec.q_sum[gp], q);
                }
                atomicAdd(&s_bc, 1ull);
              }
            }
          }
          if (bad) { atomicExch(&s_err, (int)PG_ERR_INDEX); goto next_op; }
          if (P.long_read > 0) {
            const int64_t i0 = (int64_t)dloc - g.start;  // index(dloc), used as a contig index
            if (homoRun(i0, bad) >= 4 && !bad) goto next_op;
            if (!bad && P.long_read == PG_NANOPORE) {
              bool ex = (i0 - 2 >= 0) && (i0 + 2 <= g.size - 1) && cref[i0 - 2] == 'C' && cref[i0 - 1] == 'C' &&
                        cref[i0 + 1] == 'G' && cref[i0 + 2] == 'G';
              if (ex) goto next_op;
            }
          }
          if (bad || dloc < g.start) { atomicExch(&s_err, (int)PG_ERR_INDEX); goto next_op; }
          {
            const int64_t gp = g.pos_base + (dloc - g.start);
            atomicAdd(&a.rec.mq_sum[gp], indelMq + 1);
            atomicAdd(&a.rec.del_qual[gp], indelMq + 1);
            atomicAdd(&a.rec.q_sum[gp], read_qual(R, i, readOffset, hasQual, P));
            atomicAdd(&a.rec.deletions[gp], 1);
            unsigned long long slot = atomicAdd(a.n_events, 1ull);
            if ((int64_t)slot < a.event_cap) {
              Event e;
              e.gpos = gp; e.read = i; e.region = C.region; e.len = len; e.roff = rloc;
              e.kind_rot = (int32_t)0x80000000;
              a.events[slot] = e;
            }
            atomicAdd(&a.bucket_count[g.call_tile0 + (dloc - g.start) / kCallTile], 1);
          }
        }
      next_op:
        if (op == 0 || op == 1 || op == 4 || op == 7 || op == 8) readOffset += len;
        if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) refOffset += len;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      StatsDev* st = &a.stats[C.region];
      if (s_rc) atomicAdd(&st->read_count, s_rc);
      if (s_bc) atomicAdd(&st->base_count, s_bc);
      if (s_pcs) atomicAdd(&st->phys_cov_start, s_pcs);
      if (s_iss) atomicAdd(&st->insert_size_start, s_iss);
      if (s_frc) { atomicAdd(&st->fr_count, s_frc); atomicAdd(&st->fr_sum, s_frs); atomicAdd(&st->fr_sumsq, s_frq); }
      if (s_rfc) { atomicAdd(&st->rf_count, s_rfc); atomicAdd(&st->rf_sum, s_rfs); atomicAdd(&st->rf_sumsq, s_rfq); }
      if (s_err) atomicExch(&st->error, s_err);
    }
    __syncthreads();
  }
}

void launch_read_events(const EventArgs& a, int32_t chunk_begin, int32_t chunk_count, cudaStream_t s) {
  if (chunk_count <= 0) return;
  int blocks = min(chunk_count, 152 * 8);
  k_read_events<<<blocks, 256, 0, s>>>(a, chunk_begin, chunk_begin + chunk_count);
}

// ---------------------------------------------------------------------------
// Exclusive scan of a small int32 array (n + 1 outputs) in one CTA.
__global__ void __launch_bounds__(1024) k_scan_small(const int32_t* in, int32_t* out, int32_t n) {
  __shared__ int32_t s_warp[32];
  __shared__ int32_t s_carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int32_t base = 0; base < n; base += blockDim.x) {
    int32_t i = base + threadIdx.x;
    int32_t v = i < n ? in[i] : 0;
    int32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int32_t y = __shfl_up_sync(FULL, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int32_t w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(FULL, w, o);
        if (lane >= o) w += y;
      }
      s_warp[lane] = w;
    }
    __syncthreads();
    int32_t incl = x + (warp > 0 ? s_warp[warp - 1] : 0) + s_carry;
    if (i < n) out[i] = incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry = incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = s_carry;
}

void launch_scan_small(const int32_t* in, int32_t* out_excl, int32_t n, cudaStream_t s) {
  k_scan_small<<<1, 1024, 0, s>>>(in, out_excl, n);
}

// ---------------------------------------------------------------------------
__global__ void k_event_scatter(const Event* ev, const unsigned long long* n_events, const RegionDev* regions,
                                const int32_t* bucket_off, int32_t* bucket_fill, Event* out, int64_t max_events) {
  int64_t n = min((int64_t)*n_events, max_events);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    Event e = ev[k];
    const RegionDev& g = regions[e.region];
    int32_t tile = g.call_tile0 + (int32_t)((e.gpos - g.pos_base) / kCallTile);
    int32_t slot = bucket_off[tile] + atomicAdd(&bucket_fill[tile], 1);
    if (slot < max_events) out[slot] = e;
  }
}

void launch_event_scatter(const Event* ev, const unsigned long long* n_events, const RegionDev* regions,
                          const int32_t* bucket_off, int32_t* bucket_fill, Event* out, cudaStream_t s,
                          int64_t max_events) {
  if (max_events <= 0) return;
  int blocks = (int)std::min<int64_t>((max_events + 255) / 256, 152 * 8);
  k_event_scatter<<<blocks, 256, 0, s>>>(ev, n_events, regions, bucket_off, bucket_fill, out, max_events);
}

// ---------------------------------------------------------------------------
// computePhysCov as a segmented scan over call tiles (kCallTile positions).
// Phase A: tile sums.  Phase B: per-region exclusive scan of tile sums with the
// region's start carry.  Phase C: in-tile scan, then insertSize /= physCov.
__device__ inline void block_scan_pair(uint32_t& a, uint32_t& b, uint32_t* s_a, uint32_t* s_b) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t ya = __shfl_up_sync(FULL, a, o), yb = __shfl_up_sync(FULL, b, o);
    if (lane >= o) { a += ya; b += yb; }
  }
  if (lane == 31) { s_a[warp] = a; s_b[warp] = b; }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t wa = lane < nw ? s_a[lane] : 0u, wb = lane < nw ? s_b[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t ya = __shfl_up_sync(FULL, wa, o), yb = __shfl_up_sync(FULL, wb, o);
      if (lane >= o) { wa += ya; wb += yb; }
    }
    s_a[lane] = wa; s_b[lane] = wb;
  }
  __syncthreads();
  if (warp > 0) { a += s_a[warp - 1]; b += s_b[warp - 1]; }
}

__global__ void __launch_bounds__(kCallTile) k_scan_tiles_a(const RegionDev* regions, const int32_t* tile_region,
                                                             Records rec, int32_t* tile_sums, int32_t tile_begin) {
  __shared__ uint32_t s_a[32], s_b[32];
  const int32_t t = tile_begin + blockIdx.x;
  const RegionDev& g = regions[tile_region[t]];
  const int32_t lo = (t - g.call_tile0) * kCallTile;
  const int32_t p = lo + threadIdx.x;
  uint32_t a = 0, b = 0;
  if (p < g.size) {
    a = (uint32_t)rec.phys_cov[g.pos_base + p];
    b = (uint32_t)rec.insert_size[g.pos_base + p];
  }
  block_scan_pair(a, b, s_a, s_b);
  if (threadIdx.x == blockDim.x - 1) { tile_sums[2 * t] = (int32_t)a; tile_sums[2 * t + 1] = (int32_t)b; }
}

__global__ void k_scan_tiles_b(const RegionDev* regions, int32_t n_regions, const StatsDev* stats,
                               int32_t* tile_sums) {
  int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_regions) return;
  const RegionDev& g = regions[r];
  uint32_t ca = (uint32_t)stats[r].phys_cov_start, cb = (uint32_t)stats[r].insert_size_start;
  for (int32_t t = g.call_tile0; t < g.call_tile0 + g.n_call_tiles; t++) {
    uint32_t a = (uint32_t)tile_sums[2 * t], b = (uint32_t)tile_sums[2 * t + 1];
    tile_sums[2 * t] = (int32_t)ca;
    tile_sums[2 * t + 1] = (int32_t)cb;
    ca += a;
    cb += b;
  }
}

__global__ void __launch_bounds__(kCallTile) k_scan_tiles_c(const RegionDev* regions, const int32_t* tile_region,
                                                             Records rec, const int32_t* tile_sums,
                                                             int32_t tile_begin) {
  __shared__ uint32_t s_a[32], s_b[32];
  const int32_t t = tile_begin + blockIdx.x;
  const RegionDev& g = regions[tile_region[t]];
  const int32_t lo = (t - g.call_tile0) * kCallTile;
  const int32_t p = lo + threadIdx.x;
  uint32_t a = 0, b = 0;
  if (p < g.size) {
    a = (uint32_t)rec.phys_cov[g.pos_base + p];
    b = (uint32_t)rec.insert_size[g.pos_base + p];
  }
  block_scan_pair(a, b, s_a, s_b);
  if (p < g.size) {
    int32_t pc = (int32_t)(a + (uint32_t)tile_sums[2 * t]);
    int32_t is = (int32_t)(b + (uint32_t)tile_sums[2 * t + 1]);
    if (pc > 0) is = is / pc;
    rec.phys_cov[g.pos_base + p] = pc;
    rec.insert_size[g.pos_base + p] = is;
  }
}

void launch_physcov_scan(const RegionDev* regions, const int32_t* call_tile_region, int32_t tile_begin,
                         int32_t n_tiles, Records rec, const StatsDev* stats, int32_t* tile_sums,
                         int32_t region_begin, int32_t n_regions, cudaStream_t s) {
  if (n_tiles <= 0) return;
  k_scan_tiles_a<<<n_tiles, kCallTile, 0, s>>>(regions, call_tile_region, rec, tile_sums, tile_begin);
  k_scan_tiles_b<<<(n_regions + 127) / 128, 128, 0, s>>>(regions + region_begin, n_regions, stats + region_begin,
                                                           tile_sums);
  k_scan_tiles_c<<<n_tiles, kCallTile, 0, s>>>(regions, call_tile_region, rec, tile_sums, tile_begin);
}

// ---------------------------------------------------------------------------
// minDepth of GenomeRegion.postProcess (S/GenomeRegion.scala:216-224).
__device__ inline int64_t java_round(double x) {
  double f = floor(x);
  return (int64_t)((x - f >= 0.5) ? f + 1.0 : f);
}

__global__ void k_region_prep(const RegionDev* regions, StatsDev* stats, int32_t n_regions, DevParams P) {
  int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_regions) return;
  int64_t meanCoverage = roundDivL((int64_t)stats[r].base_count, regions[r].size);
  int32_t md;
  if (P.min_depth >= 1) md = (int32_t)P.min_depth;
  else md = max((int32_t)java_round(P.min_depth * (double)meanCoverage), P.min_min_depth);
  stats[r].min_depth = md;
}

void launch_region_prep(const RegionDev* regions, StatsDev* stats, int32_t n_regions, DevParams P, cudaStream_t s) {
  if (n_regions == 0) return;
  k_region_prep<<<(n_regions + 127) / 128, 128, 0, s>>>(regions, stats, n_regions, P);
}

}  // namespace pg
