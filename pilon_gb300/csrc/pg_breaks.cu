// pg_breaks.cu — break candidates of every region of the last pileup call, on
// the device (GenomeRegion.possibleBreaks, S/GenomeRegion.scala:659-763, with
// pctBadOverall :99-114 and fragCoverage of processBam :287-300).
//
//   k_brk_frag    per position: fragCoverage = depth before the deletion-span
//                 updates of pass 1; region sums of fragCoverage, badCoverage
//                 and coverage
//   k_brk_spans   takes each accepted deletion's span update back out of
//                 fragCoverage (S/GenomeRegion.scala:259-264 adds it to depth)
//   k_brk_tiles   per position the break test (low coverage, high clipping, too
//                 many bad pairs, coverage dip) and the N test; per 1024-position
//                 tile the first and last tested position and the run starts
//                 inside the tile (summaryRegions' merge rule)
//   k_brk_merge   one warp per region: joins the tiles' runs in order, drops
//                 runs near the region's ends, keeps N runs of >= 10 bases as
//                 gaps and drops breaks near a gap (Region.near, 300 bases)
//   k_brk_compact the regions' breaks, placed by a scan of their counts: one
//                 list by region, then position
//   k_brk_windows the K-mer tally's read range of each break
#include <cuda_runtime.h>

#include "pg_breaks.cuh"

namespace pg {

#define FULL 0xffffffffu

__device__ inline bool is_del_change(uint32_t call) { return PG_CALL_CHANGE(call) == PG_CHANGE_DEL; }

__device__ inline long long block_sum(long long v, long long* s_red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s_red[warp] = v;
  __syncthreads();
  long long t = 0;
  if (warp == 0) {
    t = lane < (int)(blockDim.x >> 5) ? s_red[lane] : 0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(FULL, t, o);
  }
  return t;  // valid in thread 0
}

// kBrkThreads threads per 1024-position tile, kBrkPer consecutive positions each.
constexpr int kBrkThreads = 256;
constexpr int kBrkPer = kCallTile / kBrkThreads;

__global__ void __launch_bounds__(kBrkThreads) k_brk_frag(BreakArgs a) {
  __shared__ long long s_red[32];
  const int32_t t = a.tile_begin + blockIdx.x;
  const int32_t r = a.call_tile_region[t];
  const RegionDev g = a.regions[r];
  const int32_t p0 = (t - g.call_tile0) * kCallTile + kBrkPer * threadIdx.x;
  const bool reads = a.stats[r].read_count > 0;
  long long fr = 0, bad = 0, cov = 0;
#pragma unroll
  for (int q = 0; q < kBrkPer; q++) {
    const int32_t p = p0 + q;
    if (p < g.size) {
      const int64_t gp = g.pos_base + p;
      const int4 c = a.rec.count[gp];
      const int32_t depth = wadd(wadd(wadd(c.x, c.y), wadd(c.z, c.w)), a.rec.deletions[gp]);
      a.frag[gp] = depth;
      fr += depth;
      if (reads) {  // postProcess leaves coverage and badCoverage at 0 for a region without reads
        cov += depth;
        bad += a.rec.bad_pair[gp];
      }
    }
  }
  fr = block_sum(fr, s_red);
  if (threadIdx.x == 0) atomicAdd((unsigned long long*)&a.sums[3 * r], (unsigned long long)fr);
  bad = block_sum(bad, s_red);
  if (threadIdx.x == 0) atomicAdd((unsigned long long*)&a.sums[3 * r + 1], (unsigned long long)bad);
  cov = block_sum(cov, s_red);
  if (threadIdx.x == 0) atomicAdd((unsigned long long*)&a.sums[3 * r + 2], (unsigned long long)cov);
}

__global__ void __launch_bounds__(kCallTile) k_brk_spans(BreakArgs a) {
  const int32_t t = a.tile_begin + blockIdx.x;
  const int32_t r = a.call_tile_region[t];
  const RegionDev g = a.regions[r];
  const int32_t p = (t - g.call_tile0) * kCallTile + threadIdx.x;
  if (p >= g.size) return;
  const int64_t gp = g.pos_base + p;
  if (!is_del_change(a.rec.call[gp])) return;
  const int32_t len = a.rec.indel_len[gp], d = a.rec.deletions[gp];
  long long total = 0;
  for (int32_t k = 1; k < len && p + k < g.size; k++) {
    atomicSub(&a.frag[gp + k], d);
    total += d;
  }
  if (total) atomicAdd((unsigned long long*)&a.sums[3 * r], (unsigned long long)(-total));
}

// Exclusive max-scan over the block of v (>= -1); returns the maximum of the
// values of lower threads, -1 when none.
__device__ inline int32_t block_prev_max(int32_t v, int32_t* s_warp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(FULL, x, o);
    if (lane >= o) x = max(x, y);
  }
  const int32_t excl_in_warp = __shfl_up_sync(FULL, x, 1);
  __syncthreads();
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int32_t w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : -1;
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(FULL, w, o);
      if (lane >= o) w = max(w, y);
    }
    s_warp[lane] = w;  // inclusive maximum of warps 0..lane
  }
  __syncthreads();
  int32_t prev = warp > 0 ? s_warp[warp - 1] : -1;
  if (lane > 0) prev = max(prev, excl_in_warp);
  return prev;
}

__global__ void __launch_bounds__(kBrkThreads) k_brk_tiles(BreakArgs a) {
  __shared__ int32_t s_warp[32];
  __shared__ int32_t s_cnt[2];
  const int32_t t = a.tile_begin + blockIdx.x;
  const int32_t r = a.call_tile_region[t];
  const RegionDev g = a.regions[r];
  const int32_t p0 = (t - g.call_tile0) * kCallTile + kBrkPer * threadIdx.x;
  const int64_t base = g.pos_base;
  const bool reads = a.stats[r].read_count > 0;
  const int32_t mmd = a.min_min_depth;
  const long long sbad = a.sums[3 * r + 1], sgood = a.sums[3 * r + 2];
  const long long pbo = roundDivL(100 * sbad, sgood + sbad);
  const double mean = (double)a.sums[3 * r] / (double)g.size;
  uint32_t tb = 0, tn = 0;  // bit q: position p0 + q passes the break test / is N
#pragma unroll
  for (int q = 0; q < kBrkPer; q++) {
    const int32_t p = p0 + q;
    if (p < g.size) {
      const int64_t gp = base + p;
      uint8_t rb = a.ref[g.ref_off + g.start - 1 + p];
      if (rb >= 'a' && rb <= 'z') rb -= 32;
      const bool isN = rb == 'N';
      const int4 c = a.rec.count[gp];
      const int32_t depth = wadd(wadd(wadd(c.x, c.y), wadd(c.z, c.w)), a.rec.deletions[gp]);
      const int32_t cov = reads ? depth : 0;
      const int32_t bad = reads ? a.rec.bad_pair[gp] : 0;
      const int32_t clips = reads ? (int32_t)(int16_t)a.rec.clips[gp] : 0;  // pu.clips.toShort
      const bool lowCov = cov < mmd && !isN;
      const bool highClip = cov >= mmd && pctI(clips, cov) >= 33;
      const bool tooBad = (long long)pctI(bad, wadd(cov, bad)) > pbo + 20;
      const int32_t left = a.frag[base + max(0, p - 100)], right = a.frag[base + min(g.size - 1, p + 100)];
      const int32_t center = a.frag[gp];
      const double dipF = (double)wadd(wsub(left, center), wsub(right, center)) / mean;
      if (lowCov || highClip || tooBad || dipF >= 1.5) tb |= 1u << q;
      if (isN) tn |= 1u << q;
    }
  }
  BreakTile& T = a.tiles[t];
  if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int32_t slop = k == 0 ? 200 : 100;
    const uint32_t bits = k == 0 ? tb : tn;
    // the thread's last tested position, and the last one of the lower threads
    const int32_t mine = bits ? p0 + 31 - __clz(bits) : -1;
    int32_t prev = block_prev_max(mine, s_warp);
    const int32_t last = max(s_warp[(kBrkThreads >> 5) - 1], -1);
    // a run starts inside the tile where the previous tested position is more
    // than slop + 1 back (summaryRegions closes a run at the first untested
    // position more than slop past its last tested one)
#pragma unroll
    for (int q = 0; q < kBrkPer; q++) {
      if (!((bits >> q) & 1u)) continue;
      const int32_t p = p0 + q;
      if (prev < 0) {
        T.first[k] = p;
      } else if (p - prev > slop + 1) {
        const int j = atomicAdd(&s_cnt[k], 1);
        if (j < kBreakStarts) {
          T.start[k][j] = p;
          T.prev[k][j] = prev;
        }
      }
      prev = p;
    }
    if (threadIdx.x == 0) {
      T.last[k] = last;
      if (last < 0) T.first[k] = -1;
    }
    __syncthreads();
    if (threadIdx.x == 0) T.n[k] = min(s_cnt[k], kBreakStarts);
  }
}

// Sorts the (at most kBreakStarts) run starts of a tile, which the atomic slot
// order left unordered, in place.
__device__ inline void sort_starts(int32_t* s, int32_t* pv, int n) {
  for (int i = 1; i < n; i++) {
    const int32_t a = s[i], b = pv[i];
    int j = i - 1;
    while (j >= 0 && s[j] > a) { s[j + 1] = s[j]; pv[j + 1] = pv[j]; j--; }
    s[j + 1] = a;
    pv[j + 1] = b;
  }
}

// One warp per region: the lanes test 32 tiles at a time for runs, lane 0 joins
// the tiles that have some, in order.
__global__ void k_brk_merge(BreakArgs a, int32_t n_regions) {
  const int32_t r = (int32_t)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= n_regions) return;
  const RegionDev g = a.regions[r];
  if (a.stats[r].error) return;  // the reference threw on this region
  int2* gaps = a.gap_scratch + (int64_t)g.call_tile0 * (kBreakStarts + 1);
  int32_t n_gaps = 0, n_brk = 0;
  const int32_t tend = g.call_tile0 + g.n_call_tiles;
  // pass 0: gaps (N runs, slop 100, >= 10 bases, not near the region's ends);
  // pass 1: breaks (slop 200, not near the ends, not near a gap)
  for (int pass = 0; pass < 2; pass++) {
    const int k = pass == 0 ? 1 : 0;
    const int32_t slop = k == 0 ? 200 : 100;
    int32_t run_first = -1, carry = -1, gp_ptr = 0;
    auto emit = [&](int32_t f, int32_t l) {
      if (f < 100 || (g.size - 1 - l) < 100) return;  // nearEdge: start - region.start < 100 || stop - stop < 100
      const int32_t lf = g.start + f, ll = g.start + l;
      if (pass == 0) {
        if (ll + 1 - lf >= 10) gaps[n_gaps++] = make_int2(lf, ll);
        return;
      }
      // Region.near(gap, 300): overlap, or an end within 300 of the other region's opposite end
      while (gp_ptr < n_gaps && gaps[gp_ptr].y < lf - 300) gp_ptr++;
      for (int32_t q = gp_ptr; q < n_gaps && gaps[q].x <= ll + 300; q++) {
        const int2 G = gaps[q];
        if ((G.x <= ll && G.y >= lf) || abs(G.y - lf) <= 300 || abs(G.x - ll) <= 300) return;
      }
      a.brk_scratch[(int64_t)g.call_tile0 * (kBreakStarts + 1) + n_brk++] = make_int2(lf, ll);
    };
    for (int32_t t0 = g.call_tile0; t0 < tend; t0 += 32) {
      const int32_t tl = t0 + lane;
      unsigned m = __ballot_sync(FULL, tl < tend && a.tiles[tl].last[k] >= 0);
      if (lane == 0) {
        while (m) {
          BreakTile& T = a.tiles[t0 + __ffs(m) - 1];
          m &= m - 1;
          const int32_t f0 = T.first[k];
          if (carry < 0) run_first = f0;
          else if (f0 - carry > slop + 1) {
            emit(run_first, carry);
            run_first = f0;
          }
          const int n = T.n[k];
          sort_starts(T.start[k], T.prev[k], n);
          for (int j = 0; j < n; j++) {
            emit(run_first, T.prev[k][j]);
            run_first = T.start[k][j];
          }
          carry = T.last[k];
        }
      }
    }
    if (lane == 0 && carry >= 0) emit(run_first, carry);
    __syncwarp();
  }
  if (lane == 0) a.brk_count[r] = n_brk;
}

// One warp per region: its breaks into the region's place of the ordered list.
__global__ void k_brk_compact(BreakArgs a, int32_t n_regions) {
  const int32_t r = (int32_t)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= n_regions) return;
  const RegionDev g = a.regions[r];
  const int32_t n = a.brk_off[r + 1] - a.brk_off[r];
  const int2* src = a.brk_scratch + (int64_t)g.call_tile0 * (kBreakStarts + 1);
  for (int32_t k = lane; k < n; k += 32) a.out[a.brk_off[r] + k] = pg_break{r, src[k].x, src[k].y, 0};
}

__device__ inline int64_t lower_bound_i32(const int32_t* v, int64_t lo, int64_t hi, int64_t x) {
  while (lo < hi) {
    const int64_t m = (lo + hi) >> 1;
    if ((int64_t)v[m] < x) lo = m + 1; else hi = m;
  }
  return lo;
}

__global__ void k_brk_windows(Reads R, const RegionDev* regions, const pg_break* brk, int32_t n, int32_t radius,
                              const ReadExtent* ext, pg_window* out) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const pg_break b = brk[k];
  const RegionDev g = regions[b.region];
  // the contig's reads: ref_id is sorted
  const int64_t clo = lower_bound_i32(R.ref_id, 0, R.n, g.contig);
  const int64_t chi = lower_bound_i32(R.ref_id, clo, R.n, (int64_t)g.contig + 1);
  const int64_t qs = max((int64_t)b.start - radius, (int64_t)0);
  const int64_t qe = min((int64_t)b.stop + radius, g.contig_len);
  const int64_t a0 = lower_bound_i32(R.pos, clo, chi, qs - ext->max_span);
  const int64_t a1 = lower_bound_i32(R.pos, a0, chi, qe + 1);  // positions <= qe
  out[k] = pg_window{a0, a1};
}

void launch_breaks(const BreakArgs& a, int32_t n_regions, cudaStream_t s) {
  if (a.n_tiles <= 0) return;
  k_brk_frag<<<a.n_tiles, kBrkThreads, 0, s>>>(a);
  k_brk_spans<<<a.n_tiles, kCallTile, 0, s>>>(a);
  k_brk_tiles<<<a.n_tiles, kBrkThreads, 0, s>>>(a);
  k_brk_merge<<<(n_regions + 3) / 4, 128, 0, s>>>(a, n_regions);
  launch_scan_small(a.brk_count, a.brk_off, n_regions, s);
  k_brk_compact<<<(n_regions + 3) / 4, 128, 0, s>>>(a, n_regions);
}

// ---------------------------------------------------------------------------
// Pass 2 of GenomeRegion.postProcess (S/GenomeRegion.scala:274-283) and
// duplicationEvents (:735-741) on the fragCoverage of k_brk_frag / k_brk_spans:
//   smoothCov = smooth(fragCoverage, 200)          (S/GenomeRegion.scala:190-210)
//   copyNumber(i) = Math.round(smoothCov(i) / mean).toShort, 0 when mean <= 0
//   duplications = summaryRegions(copyNumber > 1, 2000) filter (size > 10000)
// smooth keeps the reference's arithmetic: the Int accumulator starts with
// input(0) and never drops it, so for a region of n > 200 positions
//   smoothCov(x) = (input(0) + sum input(x-99 .. x+100) + 100) / 200   for 101 <= x <= n-101,
//   smoothCov(x) = 0 for x <= 100 (result(100) is never written before it is
//   copied) and result(n-101) for x >= n-100 (0 itself when n <= 201); for
//   n <= 200 every position gets sum(input) / n.  With a merge slop of 2000
//   every tested position of a 1024-position tile belongs to one run, so each
//   tile reports its first and last tested position and one thread per region
//   joins the tiles in order.
constexpr int kDupHalo = 200;                      // positions loaded before and after a tile
constexpr int kDupSpan = kCallTile + 2 * kDupHalo;  // 1424
constexpr int kDupPer = (kDupSpan + kBrkThreads - 1) / kBrkThreads;  // 6 per thread

__global__ void __launch_bounds__(kBrkThreads) k_dup_tiles(BreakArgs a, int2* tile_runs) {
  __shared__ uint32_t s_p[kBrkThreads * kDupPer + 1];  // prefix sums of the window (wrapping Int)
  __shared__ uint32_t s_w[32];
  __shared__ int32_t s_fl[2][32];
  const int32_t t = a.tile_begin + blockIdx.x;
  const int32_t r = a.call_tile_region[t];
  const RegionDev g = a.regions[r];
  const int32_t n = g.size;
  const int32_t x0 = (t - g.call_tile0) * kCallTile;
  const int32_t w0 = x0 - kDupHalo;  // region index of window slot 0
  const bool reads = a.stats[r].read_count > 0;
  const double mean = (double)a.sums[3 * r] / (double)n;
  // prefix sums over the slots [w0, w0 + kBrkThreads * kDupPer), positions outside the region 0
  uint32_t v[kDupPer], tot = 0;
#pragma unroll
  for (int q = 0; q < kDupPer; q++) {
    const int32_t x = w0 + kDupPer * (int32_t)threadIdx.x + q;
    v[q] = (x >= 0 && x < n) ? (uint32_t)a.frag[g.pos_base + x] : 0u;
    tot += v[q];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = tot;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_w[warp] = incl;
  __syncthreads();
  uint32_t run = incl - tot;
  for (int w = 0; w < warp; w++) run += s_w[w];
#pragma unroll
  for (int q = 0; q < kDupPer; q++) {
    s_p[kDupPer * threadIdx.x + q] = run;  // sum of the slots before this one
    run += v[q];
  }
  if (threadIdx.x == kBrkThreads - 1) s_p[kBrkThreads * kDupPer] = run;
  __syncthreads();
  const uint32_t in0 = (uint32_t)a.frag[g.pos_base];
  // for n <= 200 the window holds the whole region: its input sum
  const uint32_t all = s_p[kBrkThreads * kDupPer];
  // smoothCov of region index x (101 <= x <= n - 101, n > 200): slots x - 99 .. x + 100
  auto smooth_at = [&](int32_t x) -> int32_t {
    const uint32_t win = s_p[x + 101 - w0] - s_p[x - 99 - w0];
    return (int32_t)wadd((int32_t)(in0 + win), 100) / 200;
  };
  int32_t first = -1, last = -1;
  if (reads && mean > 0) {
    for (int32_t x = x0 + threadIdx.x; x < min(x0 + kCallTile, n); x += kBrkThreads) {
      int32_t sm;
      if (n <= 200) sm = (int32_t)all / n;
      else if (x <= 100) sm = 0;
      else if (x >= n - 100) sm = n - 101 >= 101 ? smooth_at(n - 101) : 0;  // result(n-101), written when n >= 202
      else sm = smooth_at(x);
      const double y = (double)sm / mean;
      const double f = floor(y);
      const long long cn = (long long)(y - f >= 0.5 ? f + 1.0 : f);  // Math.round: ties up
      if ((int16_t)cn > 1) {
        if (first < 0) first = x;
        last = x;
      }
    }
  }
  // the tile's first and last tested index (threads hold strided positions)
  int32_t fmin = first < 0 ? INT32_MAX : first, lmax = last;
  for (int o = 16; o > 0; o >>= 1) {
    fmin = min(fmin, __shfl_down_sync(FULL, fmin, o));
    lmax = max(lmax, __shfl_down_sync(FULL, lmax, o));
  }
  if (lane == 0) { s_fl[0][warp] = fmin; s_fl[1][warp] = lmax; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int32_t f2 = INT32_MAX, l2 = -1;
    for (int w = 0; w < kBrkThreads / 32; w++) { f2 = min(f2, s_fl[0][w]); l2 = max(l2, s_fl[1][w]); }
    tile_runs[t] = make_int2(l2 < 0 ? -1 : f2, l2);
  }
}

// One thread per region: summaryRegions(copyNumber > 1, 2000) over the tiles'
// runs, then the filters !nearEdge and size > 10000; appends (region, start,
// stop) loci to out (order fixed by the host).
__global__ void k_dup_merge(BreakArgs a, int32_t n_regions, const int2* tile_runs, pg_break* out, int64_t cap,
                            unsigned long long* n_out) {
  const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_regions) return;
  const RegionDev g = a.regions[r];
  int32_t first = -1, last = -1;
  auto emit = [&]() {
    // nearEdge: within 100 of the region's ends; size = last - first + 1
    if (first >= 100 && g.size - 1 - last >= 100 && last - first + 1 > 10000) {
      const unsigned long long k = atomicAdd(n_out, 1ull);
      if ((int64_t)k < cap) out[k] = pg_break{r, g.start + first, g.start + last, 0};
    }
  };
  for (int32_t t = g.call_tile0; t < g.call_tile0 + g.n_call_tiles; t++) {
    const int2 fl = tile_runs[t];
    if (fl.y < 0) continue;
    if (last >= 0 && fl.x - last > 2001) {  // untested more than slop past the run's last tested position
      emit();
      first = -1;
    }
    if (first < 0) first = fl.x;
    last = fl.y;
  }
  if (last >= 0) emit();
}

void launch_duplications(const BreakArgs& a, int32_t n_regions, int2* tile_runs, pg_break* out, int64_t cap,
                         unsigned long long* n_out, cudaStream_t s) {
  if (a.n_tiles <= 0) return;
  k_dup_tiles<<<a.n_tiles, kBrkThreads, 0, s>>>(a, tile_runs);
  k_dup_merge<<<(n_regions + 127) / 128, 128, 0, s>>>(a, n_regions, tile_runs, out, cap, n_out);
}

void launch_break_windows(const Reads& R, const RegionDev* regions, const pg_break* brk, int32_t n,
                          int32_t radius, const ReadExtent* ext, pg_window* out, cudaStream_t s) {
  if (n <= 0) return;
  k_brk_windows<<<(n + 127) / 128, 128, 0, s>>>(R, regions, brk, n, radius, ext, out);
}

}  // namespace pg
