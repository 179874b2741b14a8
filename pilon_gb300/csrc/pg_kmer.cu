// pg_kmer.cu — hashed K-mer -> next-base tally of Assembler.addRead /
// addToPileups (S/Assembler.scala:55-87) and the edges of buildGraph
// (S/Assembler.scala:132-154), for many local-reassembly windows at once.
//
// Every window owns a power-of-two open-addressing table keyed by the 2-bit
// packed K-mer (KmerSlot: the key and the K-mer's PileUp counters in one
// 64-byte line; 128-bit keys in KmerSlotWide for K <= 63).  The host groups
// windows into batches whose tables stay in L2, so the probes and the counter
// atomics of a batch are L2 operations.  One warp walks one read: lane l takes
// the l-th 32nd of the strand's K-mer starts, primes its key with the K - 1
// bases before its first start, then rolls it one base per K-mer and adds the
// following base to the K-mer's counters with global integer atomics; forward
// strand, then reverse complement.  A probe sequence is at most kMaxProbe
// slots: a longer one marks the window full, its edges are not written, and
// the host counts it again in a table four times larger.  K-mers containing a
// base other than A/C/G/T (N, IUPAC codes, '=') cannot be 2-bit packed; they
// are tallied exactly by k_kmer_exotic, one warp per window, in a table keyed
// by the 4-bit codes of the K-mer.
#include <cuda_runtime.h>

#include "pg_internal.cuh"
#include "pg_kmer.cuh"

namespace pg {

constexpr unsigned long long kTop = 1ull << 63;  // set in every stored key
constexpr unsigned FULL = 0xffffffffu;

__device__ inline int code2(uint32_t nib) { return nib == 1 ? 0 : nib == 2 ? 1 : nib == 4 ? 2 : nib == 8 ? 3 : -1; }
__device__ inline uint32_t comp_nib(uint32_t n) {  // Bases.complement: A<->T, C<->G, others unchanged
  return n == 1 ? 8u : n == 8 ? 1u : n == 2 ? 4u : n == 4 ? 2u : n;
}
__device__ inline unsigned long long mix64(unsigned long long x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull; x ^= x >> 33;
  return x;
}
// nibble of base j of a read's strand (0 = forward, 1 = reverse complement);
// seq points at the read's first sequence byte
__device__ inline uint32_t strand_nib(const uint8_t* seq, int32_t L, int strand, int32_t j) {
  const int32_t k = strand == 0 ? j : L - 1 - j;
  const uint8_t b = seq[k >> 1];
  const uint32_t n = (k & 1) ? (b & 15u) : (uint32_t)(b >> 4);
  return strand == 0 ? n : comp_nib(n);
}
__device__ inline int32_t strand_qual(const uint8_t* qual, int32_t L, int strand, int32_t j, bool hasQual, int32_t dq) {
  if (!hasQual) return dq;
  return (int32_t)(int8_t)qual[strand == 0 ? j : L - 1 - j];
}

// Per window: reads longer than K, K-mer events and exotic K-mer events.
// rlist: when not null, a window's range indexes this list of reads.
__global__ void k_kmer_prepass(Reads R, const pg_window* wins, const int64_t* rlist, int32_t K,
                               long long* out /* 3 per window */) {
  __shared__ unsigned long long s[3];
  const pg_window w = wins[blockIdx.x];
  if (threadIdx.x < 3) s[threadIdx.x] = 0;
  __syncthreads();
  unsigned long long nr = 0, ne = 0, nx = 0;
  for (int64_t ii = w.read_begin + threadIdx.x; ii < w.read_end; ii += blockDim.x) {
    const int64_t i = rlist ? rlist[ii] : ii;
    const int32_t L = R.l_seq[i];
    if (L <= K) continue;
    nr++;
    ne += 2ull * (unsigned long long)(L - K);
    const uint8_t* seq = R.seq + R.seq_off[i];
    for (int strand = 0; strand < 2; strand++) {
      int32_t lastBad = -1;
      for (int32_t j = 0; j < L - 1; j++) {
        if (code2(strand_nib(seq, L, strand, j)) < 0) lastBad = j;
        int32_t o = j - K + 1;
        if (o >= 0 && lastBad >= o) nx++;
      }
    }
  }
  atomicAdd(&s[0], nr);
  atomicAdd(&s[1], ne);
  atomicAdd(&s[2], nx);
  __syncthreads();
  if (threadIdx.x < 3) out[3 * blockIdx.x + threadIdx.x] = (long long)s[threadIdx.x];
}

constexpr int64_t kMaxProbe = 256;
constexpr int kKmerThreads = 128;  // 4 warps, one read each at a time

// A 2-bit packed K-mer of up to 63 bases: bases in the low 2K bits of hi:lo.
struct __align__(16) Key128 {
  unsigned long long lo, hi;
};
__device__ inline bool same_key(const Key128& a, const Key128& b) { return a.lo == b.lo && a.hi == b.hi; }

// The slot of a K-mer in its window's table (inserted when absent), or -1
// when the probe sequence runs past the bound.  The narrow probe reads the key
// first and swaps only into an empty slot; keys are never removed, so a stale
// read can only be "empty", which the compare-and-swap corrects.  The wide
// probe's read is the 16-byte compare-and-swap itself, so it never sees half
// of a key.
template <bool WIDE>
__device__ __forceinline__ int64_t kmer_slot(const KmerArgs& a, int32_t w, int64_t base, int64_t cap,
                                             unsigned long long key, unsigned long long key_hi) {
  int64_t h = (int64_t)((WIDE ? mix64(key ^ mix64(key_hi)) : mix64(key)) & (unsigned long long)(cap - 1));
  const int64_t probes = cap < kMaxProbe ? cap : kMaxProbe;
  for (int64_t probe = 0; probe < probes; probe++) {
    const int64_t s = base + h;
    if (WIDE) {
      KmerSlotWide* sl = static_cast<KmerSlotWide*>(a.slots) + s;
      const Key128 kk{key, key_hi | kTop}, empty{0ull, 0ull};
      const Key128 prev = atomicCAS(reinterpret_cast<Key128*>(&sl->lo), empty, kk);
      if (same_key(prev, empty)) atomicAdd(&a.used[w], 1ull);
      if (same_key(prev, empty) || same_key(prev, kk)) return s;
    } else {
      KmerSlot* sl = static_cast<KmerSlot*>(a.slots) + s;
      const unsigned long long kk = key | kTop;
      const unsigned long long k = sl->key;
      if (k == kk) return s;
      if (k == 0ull) {
        const unsigned long long prev = atomicCAS(&sl->key, 0ull, kk);
        if (prev == 0ull) atomicAdd(&a.used[w], 1ull);
        if (prev == 0ull || prev == kk) return s;
      }
    }
    h = (h + 1) & (cap - 1);
  }
  return -1;
}

// WIDE = 0: 64-bit keys (K <= 31); WIDE = 1: 128-bit keys (K <= 63).  One warp
// per read of the CTA's chunk; lane l walks K-mer starts [l S, (l + 1) S) of
// each strand, S = ceil((L - K) / 32).
template <bool WIDE>
__global__ void __launch_bounds__(kKmerThreads) k_kmer_count(KmerArgs a) {
  const KmerChunk ch = a.chunks[blockIdx.x];
  const int32_t w = ch.w;
  if (a.full[w]) return;  // the window's table is full: it is counted again, larger, after this batch
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int32_t K = a.K;
  const unsigned long long mask = (K >= 32) ? ~0ull : ((1ull << (2 * K)) - 1);
  const unsigned long long mask_hi = (K > 32) ? ((1ull << (2 * K - 64)) - 1) : 0ull;
  const int64_t base = a.slot_base[w], cap = a.slot_cap[w];
  const int64_t xev0 = a.x_ev_base[w], xev_cap = a.x_ev_cap[w];
  const Reads& R = a.R;
  for (int64_t ii = ch.lo + warp; ii < ch.hi; ii += nwarps) {
    const int64_t i = a.rlist ? a.rlist[ii] : ii;
    const int32_t L = R.l_seq[i];
    if (L <= K) continue;
    const int32_t nev = L - K;  // K-mer starts per strand
    const int32_t per = (nev + 31) >> 5;
    const int32_t o0 = lane * per, o1 = min(o0 + per, nev);
    if (o0 >= o1) continue;
    const uint32_t mq1 = (uint32_t)R.mapq[i] + 1u;
    const uint8_t* seq = R.seq + R.seq_off[i];
    const uint8_t* qual = R.qual + R.qual_off[i];
    const bool hasQual = qual[0] != 0xFF;
    for (int strand = 0; strand < 2; strand++) {
      unsigned long long key = 0, key_hi = 0;
      int32_t lastBad = -1;
      // bases o0 .. o0 + K - 2, then one base per K-mer start
      for (int32_t j = o0; j < o0 + K - 1; j++) {
        int c = code2(strand_nib(seq, L, strand, j));
        if (c < 0) { lastBad = j; c = 0; }
        if (WIDE) key_hi = ((key_hi << 2) | (key >> 62)) & mask_hi;
        key = ((key << 2) | (unsigned long long)c) & mask;
      }
      uint32_t nib = strand_nib(seq, L, strand, o0 + K - 1);
      for (int32_t o = o0; o < o1; o++) {
        const int32_t j = o + K - 1;  // last base of the K-mer at o
        int c = code2(nib);
        if (c < 0) { lastBad = j; c = 0; }
        if (WIDE) key_hi = ((key_hi << 2) | (key >> 62)) & mask_hi;
        key = ((key << 2) | (unsigned long long)c) & mask;
        const uint32_t next = strand_nib(seq, L, strand, j + 1);
        const int bi = code2(next);
        const int32_t q = strand_qual(qual, L, strand, j + 1, hasQual, a.default_qual);
        if (bi >= 0 && q >= a.min_qual) {
          if (lastBad >= o) {
            // a K-mer with a base other than A/C/G/T: listed for k_kmer_exotic
            const unsigned long long k = atomicAdd(&a.x_ev_fill[w], 1ull);
            if ((int64_t)k < xev_cap) a.x_events[xev0 + k] = make_longlong2((long long)i, ((long long)strand << 32) | (long long)o);
            else atomicExch(a.overflow, 1);
          } else {
            const int64_t slot = kmer_slot<WIDE>(a, w, base, cap, key, key_hi);
            if (slot < 0) {
              a.full[w] = 1;  // counted again with a larger table
            } else if (WIDE) {
              KmerSlotWide* sl = static_cast<KmerSlotWide*>(a.slots) + slot;
              atomicAdd(&sl->cnt[bi], 1u);
              atomicAdd(&sl->qs[bi], (unsigned long long)((uint32_t)q * mq1));
              atomicAdd(&sl->q_sum, (uint32_t)q);
            } else {
              KmerSlot* sl = static_cast<KmerSlot*>(a.slots) + slot;
              atomicAdd(&sl->cnt[bi], 1u);
              atomicAdd(&sl->qs[bi], (unsigned long long)((uint32_t)q * mq1));
              atomicAdd(&sl->q_sum, (uint32_t)q);
            }
          }
        }
        nib = next;
      }
    }
  }
}

// BaseCall of a K-mer pileup (no indels): called base, alt base when not homozygous.
__device__ inline void kmer_call(const uint32_t cnt[4], const unsigned long long qs[4], uint32_t q_sum,
                                 int& base, int& alt) {
  int64_t c[4], v[4];
  for (int b = 0; b < 4; b++) { c[b] = cnt[b]; v[b] = (int64_t)qs[b]; }
  int o0, o1;
  if ((int32_t)q_sum > 0) order2(v, o0, o1); else order2(c, o0, o1);
  const int64_t total = v[0] + v[1] + v[2] + v[3];
  const int64_t b0 = pick4(v, o0), b1 = pick4(v, o1);
  const int64_t homoScore = b0 - (total - b0);
  const int64_t half = total / 2;
  const int64_t d1 = half - b0, d2 = half - b1;
  const int64_t hetero = total - (d1 < 0 ? -d1 : d1) - (d2 < 0 ? -d2 : d2);
  base = o0;
  alt = homoScore >= hetero ? -1 : o1;
}

// Edge k: key4 = the K-mer as 4-bit codes in four words (the narrow edge keeps
// the first two, K <= 32).
__device__ inline void store_edge(const KmerArgs& a, unsigned long long k, const unsigned long long key4[4],
                                  int32_t w, int base, int alt, int32_t depth, int32_t weight) {
  if ((int64_t)k >= a.edge_cap) return;
  if (a.wide) {
    pg_kmer_edge_wide e;
    for (int q = 0; q < 4; q++) e.key[q] = key4[q];
    e.window = w; e.next = (int8_t)base; e.alt = (int8_t)alt; e.pad_ = 0; e.depth = depth; e.weight = weight;
    a.wedges[k] = e;
  } else {
    pg_kmer_edge e;
    e.key_hi = key4[0]; e.key_lo = key4[1]; e.window = w; e.next = (int8_t)base; e.alt = (int8_t)alt; e.pad_ = 0;
    e.depth = depth; e.weight = weight;
    a.edges[k] = e;
  }
}

// kEdgeSlices CTAs per window, each over a slice of its table.
constexpr int kEdgeSlices = 16;

template <bool WIDE>
__global__ void __launch_bounds__(256) k_kmer_edges(KmerArgs a) {
  const int32_t w = a.win_list[blockIdx.x / kEdgeSlices];
  if (a.full[w]) return;
  const int64_t cap = a.slot_cap[w], per = (cap + kEdgeSlices - 1) / kEdgeSlices;
  const int64_t lo = a.slot_base[w] + (blockIdx.x % kEdgeSlices) * per;
  const int64_t hi = min(lo + per, a.slot_base[w] + cap);
  const int32_t K = a.K;
  const int lane = threadIdx.x & 31;
  // every warp runs the same number of iterations, so the whole warp meets the ballot
  for (int64_t s0 = lo; s0 < hi; s0 += blockDim.x) {
    const int64_t s = s0 + threadIdx.x;
    bool emit = false;
    uint32_t cnt[4] = {0, 0, 0, 0};
    unsigned long long key = 0, key_hi = 0;
    int32_t depth = 0;
    int b0 = 0, alt = -1;
    if (s < hi) {
      unsigned long long qs[4];
      uint32_t q_sum;
      bool used;
      if (WIDE) {
        const KmerSlotWide& sl = static_cast<const KmerSlotWide*>(a.slots)[s];
        key = sl.lo; key_hi = sl.hi & ~kTop; used = sl.hi != 0ull;
        for (int b = 0; b < 4; b++) { cnt[b] = sl.cnt[b]; qs[b] = sl.qs[b]; }
        q_sum = sl.q_sum;
      } else {
        const KmerSlot& sl = static_cast<const KmerSlot*>(a.slots)[s];
        key = sl.key & ~kTop; used = sl.key != 0ull;
        for (int b = 0; b < 4; b++) { cnt[b] = sl.cnt[b]; qs[b] = sl.qs[b]; }
        q_sum = sl.q_sum;
      }
      if (used) {
        depth = (int32_t)(cnt[0] + cnt[1] + cnt[2] + cnt[3]);
        if (depth >= a.min_depth) {
          kmer_call(cnt, qs, q_sum, b0, alt);
          emit = true;
        }
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, emit);
    if (!m) continue;
    unsigned long long first = 0;
    if (lane == __ffs(m) - 1) first = atomicAdd(a.n_edges, (unsigned long long)__popc(m));
    first = __shfl_sync(0xffffffffu, first, __ffs(m) - 1);
    if (emit) {
      // 2-bit digit of base j at bit 2 (K - 1 - j) of hi:lo -> its 4-bit code 1 << digit
      unsigned long long key4[4] = {0, 0, 0, 0};
      for (int32_t j = 0; j < K; j++) {
        const int32_t bit = 2 * (K - 1 - j);
        const unsigned long long d = bit < 64 ? (key >> bit) & 3ull : (key_hi >> (bit - 64)) & 3ull;
        key4[j >> 4] |= (1ull << d) << (60 - 4 * (j & 15));
      }
      store_edge(a, first + __popc(m & ((1u << lane) - 1u)), key4, w, b0, alt, depth,
                 (int32_t)(b0 == 0 ? cnt[0] : b0 == 1 ? cnt[1] : b0 == 2 ? cnt[2] : cnt[3]));
    }
  }
}

// Exotic K-mers: one warp per window over the window's listed events, 32 at a
// time, in the window's table keyed by 4-bit codes.  The warp owns the table,
// so it inserts without atomics or waits: the lanes look their keys up, the
// lanes whose key is absent group by key (__match_any_sync on every key word),
// and the groups' first lanes insert one after another in lane order, each
// from its hash slot to the next free one (keys inserted meanwhile differ from
// it).  Every lane then adds its next base to its key's counters with global
// atomics (the lanes of one key add to one slot).  Last, the warp reads the
// table 32 slots at a time and writes the edges.
constexpr int kExoticThreads = 128;

template <bool WIDE>
__global__ void __launch_bounds__(kExoticThreads) k_kmer_exotic(KmerArgs a, int32_t n_win) {
  constexpr int NW = WIDE ? 4 : 2;  // key words per slot
  const int lane = threadIdx.x & 31;
  const int32_t wl = (int32_t)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (wl >= n_win) return;  // the whole warp leaves
  const int32_t w = a.win_list[wl];
  const int64_t base = a.x_base[w], cap = a.x_cap[w];
  if (cap == 0 || a.full[w]) return;  // a full window is counted again, exotic K-mers included
  const int32_t K = a.K;
  const Reads& R = a.R;
  const int64_t nev = min((int64_t)a.x_ev_fill[w], a.x_ev_cap[w]);
  const int64_t ev0 = a.x_ev_base[w];
  for (int64_t k0 = 0; k0 < nev; k0 += 32) {
    const int64_t k = k0 + lane;
    const bool have = k < nev;
    unsigned long long kw[NW];
#pragma unroll
    for (int q = 0; q < NW; q++) kw[q] = 0;
    int bi = 0;
    int32_t qv = 0;
    uint32_t mq1 = 0;
    int64_t h = 0;
    if (have) {
      const longlong2 ev = a.x_events[ev0 + k];
      const int64_t i = ev.x;
      const int strand = (int)(ev.y >> 32);
      const int32_t o = (int32_t)(ev.y & 0xffffffffll);
      const int32_t L = R.l_seq[i];
      mq1 = (uint32_t)R.mapq[i] + 1u;
      const uint8_t* seq = R.seq + R.seq_off[i];
      const uint8_t* qual = R.qual + R.qual_off[i];
      const bool hasQual = qual[0] != 0xFF;
      bi = code2(strand_nib(seq, L, strand, o + K));
      qv = strand_qual(qual, L, strand, o + K, hasQual, a.default_qual);
      for (int32_t t = 0; t < K; t++) {
        const unsigned long long nb = strand_nib(seq, L, strand, o + t);
        kw[t >> 4] |= nb << (60 - 4 * (t & 15));
      }
      unsigned long long hv = 0;
#pragma unroll
      for (int q = 0; q < NW; q++) hv = mix64(hv ^ kw[q]);
      h = (int64_t)(hv & (unsigned long long)(cap - 1));
    }
    // look-up: the key's slot, or absent when the probe meets a free slot first
    int64_t slot = -1;
    bool absent = false;
    if (have) {
      int64_t hh = h;
      for (int64_t probe = 0; probe < cap; probe++) {
        const int64_t sl = base + hh;
        if (!a.x_used[sl]) { absent = true; break; }
        bool same = true;
#pragma unroll
        for (int q = 0; q < NW; q++) same = same && a.x_keys[NW * sl + q] == kw[q];
        if (same) { slot = sl; break; }
        hh = (hh + 1) & (cap - 1);
      }
    }
    const unsigned need = __ballot_sync(FULL, absent);
    if (need) {
      unsigned grp = FULL;
#pragma unroll
      for (int q = 0; q < NW; q++) grp &= __match_any_sync(FULL, kw[q]);
      grp &= need;  // for an absent lane: the absent lanes with its key, itself included
      const int first = absent ? __ffs(grp) - 1 : lane;
      unsigned leaders = __ballot_sync(FULL, absent && first == lane);
      while (leaders) {
        const int l = __ffs(leaders) - 1;
        if (lane == l) {
          int64_t hh = h;
          for (int64_t probe = 0; probe < cap; probe++) {
            const int64_t sl = base + hh;
            if (!a.x_used[sl]) {
              a.x_used[sl] = 1;
#pragma unroll
              for (int q = 0; q < NW; q++) a.x_keys[NW * sl + q] = kw[q];
              slot = sl;
              break;
            }
            hh = (hh + 1) & (cap - 1);
          }
        }
        __syncwarp();  // the inserted key is seen by the next leader's probe
        leaders &= leaders - 1;
      }
      const long long ls = __shfl_sync(FULL, (long long)slot, first);
      if (absent) slot = ls;
    }
    if (have) {
      if (slot < 0) {
        atomicExch(a.overflow, 1);
      } else {
        atomicAdd(&a.x_cnt[4 * slot + bi], 1u);
        atomicAdd(&a.x_qs[4 * slot + bi], (unsigned long long)((uint32_t)qv * mq1));
        atomicAdd(&a.x_q[slot], (uint32_t)qv);
      }
    }
    __syncwarp();
  }
  __threadfence();
  __syncwarp();
  // edges of the window's exotic K-mers, 32 slots at a time
  for (int64_t s0 = base; s0 < base + cap; s0 += 32) {
    const int64_t sl = s0 + lane;
    bool emit = false;
    uint32_t cnt[4] = {0, 0, 0, 0};
    int32_t depth = 0;
    int b0 = 0, alt = -1;
    if (sl < base + cap && a.x_used[sl]) {
      // the counters were added by atomics of this kernel: read them from L2
      unsigned long long qs[4];
      for (int b = 0; b < 4; b++) { cnt[b] = __ldcg(&a.x_cnt[4 * sl + b]); qs[b] = __ldcg(&a.x_qs[4 * sl + b]); }
      depth = (int32_t)(cnt[0] + cnt[1] + cnt[2] + cnt[3]);
      if (depth >= a.min_depth) {
        kmer_call(cnt, qs, __ldcg(&a.x_q[sl]), b0, alt);
        emit = true;
      }
    }
    const unsigned m = __ballot_sync(FULL, emit);
    if (!m) continue;
    unsigned long long e0 = 0;
    if (lane == __ffs(m) - 1) e0 = atomicAdd(a.n_edges, (unsigned long long)__popc(m));
    e0 = __shfl_sync(FULL, e0, __ffs(m) - 1);
    if (emit) {
      unsigned long long key4[4] = {0, 0, 0, 0};
#pragma unroll
      for (int q = 0; q < NW; q++) key4[q] = a.x_keys[NW * sl + q];
      store_edge(a, e0 + __popc(m & ((1u << lane) - 1u)), key4, w, b0, alt, depth,
                 (int32_t)(b0 == 0 ? cnt[0] : b0 == 1 ? cnt[1] : b0 == 2 ? cnt[2] : cnt[3]));
    }
  }
}

void launch_kmer_prepass(const Reads& R, const pg_window* wins, const int64_t* rlist, int32_t n, int32_t K,
                         long long* out,
                         cudaStream_t s) {
  if (n <= 0) return;
  k_kmer_prepass<<<n, 256, 0, s>>>(R, wins, rlist, K, out);
}

__global__ void k_kmer_reset(KmerArgs a) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n_win) return;
  const int32_t w = a.win_list[k];
  a.full[w] = 0;
  a.used[w] = 0;
  a.x_ev_fill[w] = 0;
}

void launch_kmer_reset(const KmerArgs& a, cudaStream_t s) {
  if (a.n_win <= 0) return;
  k_kmer_reset<<<(a.n_win + 127) / 128, 128, 0, s>>>(a);
}

void launch_kmer_count(const KmerArgs& a, cudaStream_t s) {
  if (a.n_win <= 0 || a.n_chunks <= 0) return;
  if (a.wide) k_kmer_count<true><<<a.n_chunks, kKmerThreads, 0, s>>>(a);
  else k_kmer_count<false><<<a.n_chunks, kKmerThreads, 0, s>>>(a);
}

void launch_kmer_exotic(const KmerArgs& a, cudaStream_t s) {
  if (a.n_win <= 0) return;
  const int32_t xg = (int32_t)(((int64_t)a.n_win * 32 + kExoticThreads - 1) / kExoticThreads);
  if (a.wide) k_kmer_exotic<true><<<xg, kExoticThreads, 0, s>>>(a, a.n_win);
  else k_kmer_exotic<false><<<xg, kExoticThreads, 0, s>>>(a, a.n_win);
}

void launch_kmer_edges(const KmerArgs& a, cudaStream_t s) {
  if (a.n_win <= 0) return;
  if (a.wide) k_kmer_edges<true><<<a.n_win * kEdgeSlices, 256, 0, s>>>(a);
  else k_kmer_edges<false><<<a.n_win * kEdgeSlices, 256, 0, s>>>(a);
}

}  // namespace pg
