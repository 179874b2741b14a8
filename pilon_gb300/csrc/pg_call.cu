// pg_call.cu — per-position calls and pass 1 of GenomeRegion.postProcess.
//
//   k_call        PileUp.baseCall for every position (S/PileUp.scala:132-255) and
//                 the pass-1 disposition (confirmed / INS / DEL / SNP / AMB,
//                 S/GenomeRegion.scala:237-272) computed on the unmodified pileups
//   k_cand_list   change candidates compacted in position order, per call tile
//   k_resolve     the sequential part of pass 1: a homozygous deletion call marks
//                 the next len-1 positions deleted, so later candidates inside an
//                 accepted deletion are dropped (one thread per region walks its
//                 sparse candidate list)
//   k_apply_spans adds the deletion's count to the pileups it covers
//                 (S/GenomeRegion.scala:261-264) and recomputes their calls
#include <cuda_runtime.h>

#include <algorithm>

#include "pg_internal.cuh"

namespace pg {

#define FULL 0xffffffffu

// n_ev = insertions + deletions of the position before any deletion-span update
__device__ inline CallCtx make_ctx(const CallArgs& a, int64_t ref_off, int64_t contig_len, int64_t gp, int32_t n_ev) {
  CallCtx c;
  c.ev = a.ev_sorted;
  c.ev_lo = c.ev_hi = 0;
  if (n_ev > 0) {
    const int64_t hi = a.rec.ev_end[gp];
    c.ev_hi = min(hi, a.event_cap);
    c.ev_lo = min(max(hi - n_ev, (int64_t)0), a.event_cap);
  }
  c.spool = a.spool;
  c.ref = a.ref;
  c.ref_off = ref_off;
  c.contig_len = contig_len;
  c.pool = a.pool;
  c.pool_fill = a.pool_fill;
  c.pool_cap = a.pool_cap;
  return c;
}

// BaseCall and the pass-1 disposition of position p of the tile's region
// (global position gp) from its record and its reference base rb; writes the
// call record and returns the change kind (0: none).
__device__ __forceinline__ uint32_t call_position(const CallArgs& a, const CallDesc& d, int32_t p, int64_t gp,
                                                  const PosRec& rec, uint8_t rb) {
  uint32_t change = 0;
  CallCtx c = make_ctx(a, d.ref_off, d.contig_len, gp, wadd(rec.insertions, rec.deletions));
  const int64_t locus0 = (int64_t)d.start - 1 + p;
  CallOut o = base_call(rec, a.P, c, gp, locus0);
  int32_t ins = -1;
  if (o.flags & PG_CALL_INS) ins = pool_insertion(c, c.ev[o.win_event]);
  uint32_t f = o.flags;
  if (d.reads) {
    const int64_t n = rec.cnt[0] + rec.cnt[1] + rec.cnt[2] + rec.cnt[3];
    const int64_t depth = n + rec.deletions;
    const bool isIns = f & PG_CALL_INS, isDel = f & PG_CALL_DEL;
    const bool called = (f & PG_CALL_HAS_BASE) || isIns || isDel;
    if (depth >= d.min_depth && rb != 'N' && called) {
      // 'A','C','G','T' are the bytes of 0x54474341
      const uint8_t b = (f & PG_CALL_HAS_BASE) ? (uint8_t)(0x54474341u >> (8 * (f & 3u))) : (uint8_t)'N';
      const uint8_t alt = (uint8_t)(0x54474341u >> (8 * ((f >> 2) & 3u)));
      const bool homo = f & PG_CALL_HOMO, homoIndel = f & PG_CALL_HOMO_INDEL;
      // highConfidence: q = score / n >= 10 (q = 0 when n = 0), i.e. score >= 10 n for n > 0
      const bool highConf = n > 0 && o.score >= 10 * n;
      if (homo && b == rb && highConf && !(isIns || isDel)) f |= PG_CALL_CONFIRMED;
      else if (isIns && homoIndel) change = PG_CHANGE_INS;
      else if (isDel && homoIndel) change = PG_CHANGE_DEL;
      else if (b != rb && o.score > 0) {
        if (homo) change = PG_CHANGE_SNP;
        else if (a.P.fix_amb || alt != rb) change = PG_CHANGE_AMB;
      }
    }
  }
  f |= change << 9;
  a.rec.call[gp] = f;
  a.rec.score[gp] = o.score;
  a.rec.indel_len[gp] = o.indel_len;
  a.rec.ins_str[gp] = ins;
  return change;
}

// One thread per call tile: the tile's descriptor (after k_region_prep).
__global__ void k_call_desc(CallArgs a, int32_t tile_begin) {
  const int32_t t = tile_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tile_begin + a.n_call_tiles) return;
  const int32_t r = a.call_tile_region[t];
  const RegionDev& g = a.regions[r];
  const StatsDev& st = a.stats[r];
  CallDesc d;
  d.p0 = (t - g.call_tile0) * kCallTile;
  d.gp0 = g.pos_base + d.p0;
  d.ref_off = g.ref_off;
  d.contig_len = g.contig_len;
  d.start = g.start;
  d.n = min(g.size - d.p0, kCallTile);
  d.min_depth = st.min_depth;
  d.reads = st.read_count > 0;
  d.pad = 0;
  a.call_desc[t] = d;
}

// k_call: one thread per position, kCallUnits CTAs of kCallThreads per call
// tile.  A thread's loads start from its tile's descriptor (one load), and the
// reference byte is loaded with the record, so every load of a position is in
// flight at once.  (A persistent form that staged the next unit's record into
// shared memory by cp.async while calling the current one ran 15% slower: the
// two stage buffers and the carried state cut residency to 19 warps per SM and
// one unit of work did not cover the load latency.)
constexpr int kCallThreads = 256;
constexpr int kCallUnits = kCallTile / kCallThreads;
static_assert(kCallUnits * kCallThreads == kCallTile, "call tile split");

__global__ void __launch_bounds__(kCallThreads, 6) k_call(CallArgs a, int32_t tile_begin) {
  const int32_t t = tile_begin + blockIdx.x / kCallUnits;
  const CallDesc d = a.call_desc[t];
  const int32_t k = (blockIdx.x % kCallUnits) * kCallThreads + threadIdx.x;  // index in the tile
  uint32_t changes = 0;
  if (k < d.n) {
    const int64_t gp = d.gp0 + k;
    PosRec rec;
    load_rec(a.rec, gp, rec);
    const uint8_t rb = upper(a.ref[d.ref_off + (int64_t)d.start - 1 + d.p0 + k]);
    changes = call_position(a, d, d.p0 + k, gp, rec, rb) != 0;
  }
  changes = __reduce_add_sync(FULL, changes);
  if ((threadIdx.x & 31) == 0 && changes) atomicAdd(&a.cand_count[t], (int32_t)changes);
}

void launch_call(const CallArgs& a, int32_t tile_begin, int32_t n_tiles, cudaStream_t s) {
  if (n_tiles <= 0) return;
  k_call_desc<<<(n_tiles + 255) / 256, 256, 0, s>>>(a, tile_begin);
  k_call<<<n_tiles * kCallUnits, kCallThreads, 0, s>>>(a, tile_begin);
}

// The change candidates of a call tile in position order, at the tile's offset
// from the scan of k_call's per-tile counts.  256 threads per 1024-position
// tile: the call words are loaded coalesced into shared memory, each thread
// ranks four consecutive positions, and a block scan joins the threads.
constexpr int kCandThreads = 256;
__global__ void __launch_bounds__(kCandThreads) k_cand_list(CallArgs a, const int32_t* cand_off, Cand* cands,
                                                             int32_t cand_cap, int32_t tile_begin) {
  __shared__ __align__(16) uint32_t s_k[kCallTile];
  __shared__ int32_t s_w[kCandThreads / 32];
  const int32_t t = tile_begin + blockIdx.x;
  if (a.cand_count[t] == 0) return;  // k_call counted the tile's changes: none (the whole CTA leaves)
  const int32_t r = a.call_tile_region[t];
  const RegionDev g = a.regions[r];
  const int32_t p0 = (t - g.call_tile0) * kCallTile;
  const int32_t n = min(kCallTile, g.size - p0);
  for (int32_t i = threadIdx.x; i < kCallTile; i += kCandThreads)
    s_k[i] = i < n ? PG_CALL_CHANGE(a.rec.call[g.pos_base + p0 + i]) : 0u;
  __syncthreads();
  const uint4 k4 = reinterpret_cast<const uint4*>(s_k)[threadIdx.x];  // positions 4 tid .. 4 tid + 3
  const uint32_t kk[4] = {k4.x, k4.y, k4.z, k4.w};
  const int32_t mine = (k4.x != 0) + (k4.y != 0) + (k4.z != 0) + (k4.w != 0);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_w[warp] = incl;
  __syncthreads();
  int32_t before = incl - mine;
  for (int w = 0; w < warp; w++) before += s_w[w];
  if (mine) {
    int32_t slot = cand_off[t] + before;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      if (!kk[j]) continue;
      const int32_t p = p0 + 4 * (int32_t)threadIdx.x + j;
      const int64_t gp = g.pos_base + p;
      Cand c;
      c.gpos = gp;
      c.region = r;
      c.p = p;
      c.kind = (int32_t)kk[j];
      c.len = a.rec.indel_len[gp];
      if (slot < cand_cap) cands[slot] = c;
      slot++;
    }
  }
}

// The changes of every call tile (final call flags), for pg_fetch_changes:
// k_change_count counts a tile's changes, k_change_write places them at the
// tile's offset from the scan of the counts, in position order.
__global__ void __launch_bounds__(kCandThreads) k_change_count(const RegionDev* regions, const int32_t* tile_region,
                                                                const uint32_t* call, int32_t* count) {
  __shared__ int32_t s_w[kCandThreads / 32];
  const int32_t t = blockIdx.x;
  const RegionDev& g = regions[tile_region[t]];
  const int32_t p0 = (t - g.call_tile0) * kCallTile;
  int32_t n = 0;
  for (int32_t i = threadIdx.x; i < kCallTile; i += kCandThreads)
    if (p0 + i < g.size) n += PG_CALL_CHANGE(call[g.pos_base + p0 + i]) != 0;
  n = __reduce_add_sync(FULL, n);
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int32_t v = 0;
    for (int w = 0; w < kCandThreads / 32; w++) v += s_w[w];
    count[t] = v;
  }
}

__global__ void __launch_bounds__(kCandThreads) k_change_write(const RegionDev* regions, const int32_t* tile_region,
                                                                Records rec, const int32_t* count, const int32_t* off,
                                                                pg_change* out) {
  __shared__ __align__(16) uint32_t s_c[kCallTile];
  __shared__ int32_t s_w[kCandThreads / 32];
  const int32_t t = blockIdx.x;
  if (count[t] == 0) return;  // the whole CTA leaves
  const int32_t r = tile_region[t];
  const RegionDev g = regions[r];
  const int32_t p0 = (t - g.call_tile0) * kCallTile;
  const int32_t n = min(kCallTile, g.size - p0);
  for (int32_t i = threadIdx.x; i < kCallTile; i += kCandThreads) s_c[i] = i < n ? rec.call[g.pos_base + p0 + i] : 0u;
  __syncthreads();
  const uint4 c4 = reinterpret_cast<const uint4*>(s_c)[threadIdx.x];  // positions 4 tid .. 4 tid + 3
  const uint32_t cc[4] = {c4.x, c4.y, c4.z, c4.w};
  int32_t mine = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) mine += PG_CALL_CHANGE(cc[j]) != 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_w[warp] = incl;
  __syncthreads();
  int32_t slot = off[t] + incl - mine;
  for (int w = 0; w < warp; w++) slot += s_w[w];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    if (!PG_CALL_CHANGE(cc[j])) continue;
    const int32_t p = p0 + 4 * (int32_t)threadIdx.x + j;
    const int64_t gp = g.pos_base + p;
    pg_change ch;
    ch.region = r;
    ch.locus = g.start + p;
    ch.call = cc[j];
    ch.indel_len = rec.indel_len[gp];
    ch.ins_str = rec.ins_str[gp];
    ch.pad_ = 0;
    out[slot++] = ch;
  }
}

void launch_change_count(const RegionDev* regions, const int32_t* tile_region, const uint32_t* call, int32_t* count,
                         int32_t n_tiles, cudaStream_t s) {
  if (n_tiles > 0) k_change_count<<<n_tiles, kCandThreads, 0, s>>>(regions, tile_region, call, count);
}

void launch_change_write(const RegionDev* regions, const int32_t* tile_region, const Records& rec,
                         const int32_t* count, const int32_t* off, pg_change* out, int32_t n_tiles, cudaStream_t s) {
  if (n_tiles > 0) k_change_write<<<n_tiles, kCandThreads, 0, s>>>(regions, tile_region, rec, count, off, out);
}

void launch_cand_list(const CallArgs& a, const int32_t* cand_off, Cand* cands, int32_t cand_cap,
                      int32_t tile_begin, int32_t n_tiles, cudaStream_t s) {
  if (n_tiles <= 0) return;
  k_cand_list<<<n_tiles, kCandThreads, 0, s>>>(a, cand_off, cands, cand_cap, tile_begin);
}

// Pass 1 is a left-to-right scan: a candidate inside an earlier accepted
// homozygous deletion is skipped (`!deleted(i)`).  Only deletions can suppress
// later candidates, so one warp per region walks the region's candidates 32 at
// a time and decides the (sparse) deletion candidates in order; rejected ones
// get kind < 0.  n_changes starts at the candidate count; k_apply_spans
// subtracts the candidates that fall inside accepted deletions.
__global__ void k_resolve(const RegionDev* regions, int32_t n_regions, const int32_t* cand_off, Cand* cands,
                          int32_t cand_cap, StatsDev* stats) {
  const int32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= n_regions) return;
  const RegionDev& g = regions[r];
  if (g.n_call_tiles == 0) return;
  const int32_t lo = cand_off[g.call_tile0], hi = min(cand_off[g.call_tile0 + g.n_call_tiles], cand_cap);
  int32_t lastEnd = -1;
  for (int32_t base = lo; base < hi; base += 32) {
    const int32_t k = base + lane;
    int32_t p = 0, len = 0;
    bool isDel = false;
    if (k < hi) {
      const Cand c = cands[k];
      isDel = c.kind == PG_CHANGE_DEL;
      p = c.p;
      len = c.len;
    }
    unsigned m = __ballot_sync(FULL, isDel);
    while (m) {
      const int j = __ffs(m) - 1;
      m &= m - 1;
      const int32_t pj = __shfl_sync(FULL, p, j), lj = __shfl_sync(FULL, len, j);
      const bool accept = pj > lastEnd;
      if (lane == j && !accept) cands[k].kind = -PG_CHANGE_DEL;
      if (accept) lastEnd = pj + lj - 1;
    }
  }
  if (lane == 0) stats[r].n_changes = max(hi - lo, 0);
}

void launch_resolve(const RegionDev* regions, int32_t n_regions, const int32_t* cand_off, Cand* cands,
                    int32_t cand_cap, StatsDev* stats, cudaStream_t s) {
  if (n_regions == 0) return;
  k_resolve<<<(n_regions + 3) / 4, 128, 0, s>>>(regions, n_regions, cand_off, cands, cand_cap, stats);
}

__global__ void k_apply_spans(CallArgs a, const Cand* cands, const int32_t* cand_total, int32_t cand_cap) {
  const int32_t n = min(*cand_total, cand_cap);
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const Cand c = cands[k];
    if (c.kind != PG_CHANGE_DEL) continue;
    const RegionDev g = a.regions[c.region];
    const int32_t d = a.rec.deletions[c.gpos];
    int32_t removed = 0;
    for (int32_t j = 1; j < c.len; j++) {
      const int32_t p = c.p + j;
      if (p >= g.size) break;
      const int64_t gp = g.pos_base + p;
      const int32_t del0 = a.rec.deletions[gp];
      a.rec.deletions[gp] = wadd(del0, d);
      PosRec rec;
      load_rec(a.rec, gp, rec);
      CallCtx cx = make_ctx(a, g.ref_off, g.contig_len, gp, wadd(rec.insertions, del0));
      CallOut o = base_call(rec, a.P, cx, gp, (int64_t)g.start - 1 + p);
      const uint32_t old = a.rec.call[gp];
      if (PG_CALL_CHANGE(old)) removed++;
      int32_t ins = -1;
      if (o.flags & PG_CALL_INS) ins = (old & PG_CALL_INS) ? a.rec.ins_str[gp] : pool_insertion(cx, cx.ev[o.win_event]);
      a.rec.call[gp] = o.flags | PG_CALL_DELETED;
      a.rec.score[gp] = o.score;
      a.rec.indel_len[gp] = o.indel_len;
      a.rec.ins_str[gp] = ins;
    }
    if (removed) atomicSub(&a.stats[c.region].n_changes, removed);
  }
}

void launch_apply_spans(const CallArgs& a, const Cand* cands, const int32_t* cand_total, int32_t cand_cap,
                        cudaStream_t s) {
  if (cand_cap <= 0) return;
  int blocks = std::min((cand_cap + 127) / 128, 152 * 4);
  k_apply_spans<<<blocks, 128, 0, s>>>(a, cands, cand_total, cand_cap);
}

}  // namespace pg
