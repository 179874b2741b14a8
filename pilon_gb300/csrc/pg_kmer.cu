// pg_kmer.cu — hashed K-mer -> next-base tally of Assembler.addRead /
// addToPileups (S/Assembler.scala:55-87) and the edges of buildGraph
// (S/Assembler.scala:132-154), for many local-reassembly windows at once.
//
// Every window owns a power-of-two open-addressing table keyed by the 2-bit
// packed K-mer (K <= 31, so the all-ones word marks an empty slot); the host
// groups windows into batches of tables.  One thread walks one read (several
// CTAs per window, each a chunk of its reads), forward strand then reverse
// complement, and for each K-mer adds the following base into the K-mer's
// PileUp counters with global integer atomics (count[4], qualSum[4], mqSum,
// qSum).  A probe sequence is at most kMaxProbe slots: a longer one marks the
// window full and the host counts it again in a table four times larger.  K-mers containing a
// base other than A/C/G/T (N, IUPAC codes, '=') cannot be 2-bit packed; they
// are tallied exactly by k_kmer_exotic, one thread per window, in a private
// table keyed by the 4-bit codes of the K-mer.
#include <cuda_runtime.h>

#include "pg_internal.cuh"
#include "pg_kmer.cuh"

namespace pg {

constexpr unsigned long long kEmpty = ~0ull;

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
__global__ void k_kmer_prepass(Reads R, const pg_window* wins, int32_t K, long long* out /* 3 per window */) {
  __shared__ unsigned long long s[3];
  const pg_window w = wins[blockIdx.x];
  if (threadIdx.x < 3) s[threadIdx.x] = 0;
  __syncthreads();
  unsigned long long nr = 0, ne = 0, nx = 0;
  for (int64_t i = w.read_begin + threadIdx.x; i < w.read_end; i += blockDim.x) {
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

// A 2-bit packed K-mer of up to 63 bases (the wide tables): bases in the low
// 2K bits of hi:lo, so hi < 2^62 and the all-ones key marks an empty slot.
struct __align__(16) Key128 {
  unsigned long long lo, hi;
};
__device__ inline bool same_key(const Key128& a, const Key128& b) { return a.lo == b.lo && a.hi == b.hi; }

// WIDE = 0: 64-bit keys (K <= 31); WIDE = 1: 128-bit keys (K <= 63), inserted
// with the 16-byte compare-and-swap of sm_90 and later (the compare-and-swap is
// also the probe's read, so a probe never sees half of a key).
template <bool WIDE>
__global__ void __launch_bounds__(64) k_kmer_count(KmerArgs a) {
  const KmerChunk ch = a.chunks[blockIdx.x];
  const int32_t w = ch.w;
  const int32_t K = a.K;
  const unsigned long long mask = (K >= 32) ? ~0ull : ((1ull << (2 * K)) - 1);
  const unsigned long long mask_hi = (K > 32) ? ((1ull << (2 * K - 64)) - 1) : 0ull;
  Key128* const keys2 = reinterpret_cast<Key128*>(a.keys);
  const int64_t base = a.slot_base[w], cap = a.slot_cap[w];
  const int64_t xev0 = a.x_ev_base[w], xev_cap = a.x_ev_cap[w];
  const Reads& R = a.R;
  for (int64_t i = ch.lo + threadIdx.x; i < ch.hi; i += blockDim.x) {
    const int32_t L = R.l_seq[i];
    if (L <= K) continue;
    const uint32_t mq1 = (uint32_t)R.mapq[i] + 1u;
    const uint8_t* seq = R.seq + R.seq_off[i];
    const uint8_t* qual = R.qual + R.qual_off[i];
    const bool hasQual = qual[0] != 0xFF;
    for (int strand = 0; strand < 2; strand++) {
      unsigned long long key = 0, key_hi = 0;
      int32_t lastBad = -1;
      uint32_t nib = strand_nib(seq, L, strand, 0);
      for (int32_t j = 0; j < L - 1; j++) {
        int c = code2(nib);
        if (c < 0) { lastBad = j; c = 0; }
        if (WIDE) key_hi = ((key_hi << 2) | (key >> 62)) & mask_hi;
        key = ((key << 2) | (unsigned long long)c) & mask;
        const uint32_t next = strand_nib(seq, L, strand, j + 1);
        const int32_t o = j - K + 1;
        if (o >= 0) {
          const int bi = code2(next);
          const int32_t q = strand_qual(qual, L, strand, j + 1, hasQual, a.default_qual);
          if (bi >= 0 && q >= a.min_qual) {
            if (lastBad >= o) {
              // a K-mer with a base other than A/C/G/T: listed for k_kmer_exotic
              const unsigned long long k = atomicAdd(&a.x_ev_fill[w], 1ull);
              if ((int64_t)k < xev_cap) a.x_events[xev0 + k] = make_longlong2((long long)i, ((long long)strand << 32) | (long long)o);
              else atomicExch(a.overflow, 1);
            } else {
              int64_t h = (int64_t)((WIDE ? mix64(key ^ mix64(key_hi)) : mix64(key)) & (unsigned long long)(cap - 1));
              int64_t slot = -1;
              const int64_t probes = cap < kMaxProbe ? cap : kMaxProbe;
              for (int64_t probe = 0; probe < probes; probe++) {
                const int64_t s = base + h;
                if (WIDE) {
                  const Key128 kk{key, key_hi}, empty{kEmpty, kEmpty};
                  const Key128 prev = atomicCAS(&keys2[s], empty, kk);
                  if (same_key(prev, empty)) atomicAdd(&a.used[w], 1ull);
                  if (same_key(prev, empty) || same_key(prev, kk)) { slot = s; break; }
                } else {
                  unsigned long long k = a.keys[s];
                  if (k == key) { slot = s; break; }
                  if (k == kEmpty) {
                    unsigned long long prev = atomicCAS(&a.keys[s], kEmpty, key);
                    if (prev == kEmpty) atomicAdd(&a.used[w], 1ull);
                    if (prev == kEmpty || prev == key) { slot = s; break; }
                  }
                }
                h = (h + 1) & (cap - 1);
              }
              if (slot < 0) {
                a.full[w] = 1;  // counted again with a larger table
              } else {
                atomicAdd(&a.cnt[4 * slot + bi], 1u);
                atomicAdd(&a.qs[4 * slot + bi], (unsigned long long)((uint32_t)q * mq1));
                atomicAdd(&a.mq_sum[slot], mq1);
                atomicAdd(&a.q_sum[slot], (uint32_t)q);
              }
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

template <bool WIDE>
__global__ void k_kmer_edges(KmerArgs a) {
  const int32_t w = a.win_begin + blockIdx.x;
  const Key128* const keys2 = reinterpret_cast<const Key128*>(a.keys);
  const int64_t base = a.slot_base[w], cap = a.slot_cap[w];
  const int32_t K = a.K;
  const int lane = threadIdx.x & 31;
  // every warp runs the same number of iterations, so the whole warp meets the ballot
  for (int64_t s0 = base; s0 < base + cap; s0 += blockDim.x) {
    const int64_t s = s0 + threadIdx.x;
    bool emit = false;
    uint32_t cnt[4] = {0, 0, 0, 0};
    unsigned long long key = kEmpty, key_hi = kEmpty;
    int32_t depth = 0;
    int b0 = 0, alt = -1;
    if (s < base + cap) {
      if (WIDE) {
        const Key128 k2 = keys2[s];
        key = k2.lo;
        key_hi = k2.hi;
      } else {
        key = a.keys[s];
      }
      if (key != kEmpty || key_hi != kEmpty) {
        unsigned long long qs[4];
        for (int b = 0; b < 4; b++) { cnt[b] = a.cnt[4 * s + b]; qs[b] = a.qs[4 * s + b]; }
        depth = (int32_t)(cnt[0] + cnt[1] + cnt[2] + cnt[3]);
        if (depth >= a.min_depth) {
          kmer_call(cnt, qs, a.q_sum[s], b0, alt);
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

// Exotic K-mers: one thread per window over the window's listed events, in a
// private table keyed by 4-bit codes.
template <bool WIDE>
__global__ void k_kmer_exotic(KmerArgs a, int32_t n_win) {
  constexpr int NW = WIDE ? 4 : 2;  // key words per slot
  const int32_t wl = blockIdx.x * blockDim.x + threadIdx.x;
  if (wl >= n_win) return;
  const int32_t w = a.win_begin + wl;
  const int64_t base = a.x_base[w], cap = a.x_cap[w];
  if (cap == 0) return;
  const int32_t K = a.K;
  const Reads& R = a.R;
  const int64_t nev = min((int64_t)a.x_ev_fill[w], a.x_ev_cap[w]);
  for (int64_t k = 0; k < nev; k++) {
    const longlong2 ev = a.x_events[a.x_ev_base[w] + k];
    const int64_t i = ev.x;
    const int strand = (int)(ev.y >> 32);
    const int32_t o = (int32_t)(ev.y & 0xffffffffll);
    const int32_t L = R.l_seq[i];
    const uint32_t mq1 = (uint32_t)R.mapq[i] + 1u;
    const uint8_t* seq = R.seq + R.seq_off[i];
    const uint8_t* qual = R.qual + R.qual_off[i];
    const bool hasQual = qual[0] != 0xFF;
    const int bi = code2(strand_nib(seq, L, strand, o + K));
    const int32_t q = strand_qual(qual, L, strand, o + K, hasQual, a.default_qual);
    unsigned long long kw[NW];
#pragma unroll
    for (int q = 0; q < NW; q++) kw[q] = 0;
    for (int32_t t = 0; t < K; t++) {
      const unsigned long long nb = strand_nib(seq, L, strand, o + t);
      kw[t >> 4] |= nb << (60 - 4 * (t & 15));
    }
    unsigned long long hv = 0;
#pragma unroll
    for (int q = 0; q < NW; q++) hv = mix64(hv ^ kw[q]);
    int64_t h = (int64_t)(hv & (unsigned long long)(cap - 1));
    int64_t slot = -1;
    for (int64_t probe = 0; probe < cap; probe++) {
      const int64_t s = base + h;
      bool same = a.x_used[s] != 0;
#pragma unroll
      for (int q = 0; q < NW; q++) same = same && a.x_keys[NW * s + q] == kw[q];
      if (same) { slot = s; break; }
      if (!a.x_used[s]) {
        a.x_used[s] = 1;
#pragma unroll
        for (int q = 0; q < NW; q++) a.x_keys[NW * s + q] = kw[q];
        slot = s;
        break;
      }
      h = (h + 1) & (cap - 1);
    }
    if (slot < 0) { atomicExch(a.overflow, 1); continue; }
    a.x_cnt[4 * slot + bi] += 1u;
    a.x_qs[4 * slot + bi] += (unsigned long long)((uint32_t)q * mq1);
    a.x_mq[slot] += mq1;
    a.x_q[slot] += (uint32_t)q;
  }
  for (int64_t s = base; s < base + cap; s++) {
    if (!a.x_used[s]) continue;
    uint32_t cnt[4];
    unsigned long long qs[4];
    for (int b = 0; b < 4; b++) { cnt[b] = a.x_cnt[4 * s + b]; qs[b] = a.x_qs[4 * s + b]; }
    const int32_t depth = (int32_t)(cnt[0] + cnt[1] + cnt[2] + cnt[3]);
    if (depth < a.min_depth) continue;
    int b0, alt;
    kmer_call(cnt, qs, a.x_q[s], b0, alt);
    unsigned long long key4[4] = {0, 0, 0, 0};
#pragma unroll
    for (int q = 0; q < NW; q++) key4[q] = a.x_keys[NW * s + q];
    store_edge(a, atomicAdd(a.n_edges, 1ull), key4, w, b0, alt, depth,
               (int32_t)(b0 == 0 ? cnt[0] : b0 == 1 ? cnt[1] : b0 == 2 ? cnt[2] : cnt[3]));
  }
}

void launch_kmer_prepass(const Reads& R, const pg_window* wins, int32_t n, int32_t K, long long* out,
                         cudaStream_t s) {
  if (n <= 0) return;
  k_kmer_prepass<<<n, 256, 0, s>>>(R, wins, K, out);
}

void launch_kmer_count(const KmerArgs& a, int32_t n_win, cudaStream_t s) {
  if (n_win <= 0) return;
  if (a.wide) {
    if (a.n_chunks > 0) k_kmer_count<true><<<a.n_chunks, 64, 0, s>>>(a);
    k_kmer_exotic<true><<<(n_win + 63) / 64, 64, 0, s>>>(a, n_win);
  } else {
    if (a.n_chunks > 0) k_kmer_count<false><<<a.n_chunks, 64, 0, s>>>(a);
    k_kmer_exotic<false><<<(n_win + 63) / 64, 64, 0, s>>>(a, n_win);
  }
}

void launch_kmer_edges(const KmerArgs& a, int32_t n_win, cudaStream_t s) {
  if (n_win <= 0) return;
  if (a.wide) k_kmer_edges<true><<<n_win, 256, 0, s>>>(a);
  else k_kmer_edges<false><<<n_win, 256, 0, s>>>(a);
}

}  // namespace pg
