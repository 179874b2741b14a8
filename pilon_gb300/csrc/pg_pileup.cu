// pg_pileup.cu — pileup construction kernels.
//
//   k_read_extent   maxima of how far a read's walk reaches around its start
//   k_tile_ranges   per walk tile: the range of (position-sorted) reads that can touch it
//   k_walk          the CIGAR walk of PileUpRegion.addRead for M/=/X and S operators
//                   (S/PileUpRegion.scala:145-216): one CTA owns a tile of positions,
//                   accumulates PileUp.add / badPair / clips with shared-memory
//                   integer atomics and writes the tile's records once
//   k_read_events   per (region, read): BamFile.process bookkeeping (readCount,
//                   addInsert) and physCovIncr; lists the reads with I/D operators
//   k_read_indels   per listed read: the I/D operators with their left shift
//                   (S/PileUpRegion.scala:150-183), applied with global atomics after
//                   k_walk and logged as events for the indel vote
//   k_event_scatter events -> grouped by position (offsets from the scan)
//   k_scan_*        computePhysCov (S/PileUpRegion.scala:90-100) as a segmented scan
#include <cuda_runtime.h>

#include <algorithm>

#include "pg_internal.cuh"
#include "pg_format.cuh"

namespace pg {

#define FULL 0xffffffffu

__device__ inline bool consumes_read(int op) { return op == 0 || op == 1 || op == 4 || op == 7 || op == 8; }
__device__ inline bool consumes_ref(int op) { return op == 0 || op == 2 || op == 3 || op == 7 || op == 8; }

// validateRead (S/BamFile.scala:101-105)
__device__ inline bool validate_read(uint16_t fl, const DevParams& P) {
  return (P.nonpf || !(fl & 0x200)) && (P.duplicates || !(fl & 0x400)) && !(fl & 0x100);
}

// ---------------------------------------------------------------------------
// Also validates the store: every read's CIGAR, bases and qualities must lie
// inside their arrays, and positions must not decrease within a reference.
__global__ void k_read_extent(Reads R, ReadExtent* out, int4* desc) {
  int32_t lead = 0, back = 0, span = 0;
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
      if (i > 0) {
        const int32_t r0 = R.ref_id[i - 1], r1 = R.ref_id[i];
        if (r1 == r0 && pos < R.pos[i - 1]) out->unsorted = 1;
        if ((r0 < 0 && r1 >= 0) || (r1 >= 0 && r1 < r0)) out->ungrouped = 1;
      }
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
    span = max(span, (int32_t)min((long long)R.aend[i] - pos + 1, (long long)(1 << 30)));
    back = max(back, (int32_t)min((long long)(hi - pos), (long long)(1 << 30)));
    // the walk descriptor (the shape tests of PileUpRegion.addRead's CIGAR walk,
    // S/PileUpRegion.scala:139-145, with the same int32 arithmetic as the walk)
    {
      const uint16_t fl = R.flag[i];
      const int32_t length = R.l_seq[i], mq = R.mapq[i];
      int32_t clipped = 0, ld = 0, tr = 0, nM = 0, mlen = 0, wlo = pos, whi = pos - 1, r2 = 0, f2 = 0;
      bool simple = true, indel = false;
      for (int k = 0; k < nc; k++) {
        const uint32_t w = R.cigar[co + k];
        const int32_t ln = (int32_t)(w >> 4);
        const int op = (int)(w & 15u);
        const int32_t locus = pos + f2;
        if (op == 4) {
          clipped += ln;
          const int32_t cs = r2 == 0 ? locus - ln : locus;
          wlo = min(wlo, cs);
          whi = max(whi, cs + ln - 1);
          if (nM == 0) { if (ld) simple = false; ld = ln; }
          else { if (tr) simple = false; tr = ln; }
        } else if (op == 0 || op == 7 || op == 8) {
          if (nM || tr) simple = false;
          nM++;
          mlen = ln;
          wlo = min(wlo, locus);
          whi = max(whi, locus + ln - 1);
        } else if (op != 5) {
          simple = false;
          if (op == 1 || op == 2) indel = true;
        }
        if (consumes_read(op)) r2 += ln;
        if (consumes_ref(op)) f2 += ln;
      }
      const int32_t adjMq = roundDivI(wmul(mq, length - clipped), length);
      if (nM == 0 || ld > 0xffff || tr >= 0xffff || adjMq < 0 || adjMq > 255 || mlen >= (1 << 30)) simple = false;
      const bool hasQual = length > 0 && R.qual[R.qual_off[i]] != 0xFF;
      const bool pairOk = !(fl & 0x1) || ((fl & 0x2) && R.ref_id[i] == R.mate_ref_id[i]);
      const int32_t lrel = (int32_t)min((long long)pos - wlo, (long long)((1 << 30) - 1));
      desc[2 * i] = make_int4(pos, (fl & 0x4) ? pos : R.aend[i], R.ref_id[i], adjMq + 1);
      desc[2 * i + 1] = make_int4(
          simple ? (int32_t)((uint32_t)ld | ((uint32_t)tr << 16)) : (indel ? 1 : 0),
          (int32_t)((simple ? (uint32_t)mlen : 0u) | (hasQual ? kDescHasQual : 0u) | (simple ? kDescSimple : 0u)),
          (int32_t)((uint32_t)lrel | (pairOk ? kDescPairOk : 0u)), whi - pos);
      // histogram of adjMq + 1 over the reads the walk's fast path takes, one
      // atomic per distinct value in the warp
      const uint32_t bin = (simple && hasQual) ? (uint32_t)(adjMq + 1) : 0u;
      const unsigned act = __activemask();
      const unsigned peers = __match_any_sync(act, bin);
      if (bin && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&out->mq1_hist[bin], (unsigned)__popc(peers));
    }
  }
  lead = __reduce_max_sync(FULL, lead);
  back = __reduce_max_sync(FULL, back);
  span = __reduce_max_sync(FULL, span);
  for (int o = 16; o > 0; o >>= 1) nid += __shfl_down_sync(FULL, nid, o);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out->max_lead, lead);
    atomicMax(&out->max_back, back);
    atomicMax(&out->max_span, span);
    atomicAdd(&out->n_indel_ops, nid);
  }
}

void launch_read_extent(const Reads& R, ReadExtent* out, int4* desc, cudaStream_t s) {
  cudaMemsetAsync(out, 0, sizeof(ReadExtent), s);
  if (R.n == 0) return;
  int blocks = (int)std::min<int64_t>((R.n + 255) / 256, 152 * 16);
  k_read_extent<<<blocks, 256, 0, s>>>(R, out, desc);
}

// ---------------------------------------------------------------------------
// A packed read store: each read's CIGAR words, base bytes and qualities follow
// the previous read's, so their offsets are prefix sums of the lengths, and
// the alignment end (htsjdk getAlignmentEnd: 0 for an unmapped read, else pos
// plus the reference-consuming lengths minus 1) follows from the CIGAR.
__global__ void k_packed_lengths(Reads R, int64_t* cig, int64_t* seq, int64_t* qual) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < R.n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t L = R.l_seq[i];
    cig[i] = R.n_cigar[i];
    seq[i] = ((int64_t)L + 1) / 2;
    qual[i] = L;
  }
}

__global__ void k_packed_aend(Reads R, int32_t* aend) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < R.n; i += (int64_t)gridDim.x * blockDim.x) {
    if (R.flag[i] & 0x4) { aend[i] = 0; continue; }
    const int64_t co = R.cigar_off[i];
    const int nc = R.n_cigar[i];
    int64_t reflen = 0;
    for (int k = 0; k < nc; k++) {
      const uint32_t w = R.cigar[co + k], op = w & 15u;
      if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) reflen += w >> 4;
    }
    aend[i] = (int32_t)((uint32_t)R.pos[i] + (uint32_t)reflen - 1u);  // Java int arithmetic: wraps
  }
}

void launch_packed_lengths(const Reads& R, int64_t* cig, int64_t* seq, int64_t* qual, cudaStream_t s) {
  if (R.n <= 0) return;
  k_packed_lengths<<<(int)std::min<int64_t>((R.n + 255) / 256, 152 * 16), 256, 0, s>>>(R, cig, seq, qual);
}

void launch_packed_aend(const Reads& R, int32_t* aend, cudaStream_t s) {
  if (R.n <= 0) return;
  k_packed_aend<<<(int)std::min<int64_t>((R.n + 255) / 256, 152 * 16), 256, 0, s>>>(R, aend);
}

// ---------------------------------------------------------------------------
// Walk entries: one per M/=/X or S operator (the operators whose bases the walk
// adds, S/PileUpRegion.scala:184-206), with everything of the read the walk
// needs beside it, so that a walk tile reads its entries as one coalesced
// stream and never interprets a CIGAR.
__device__ inline bool entry_op(int op) { return op == 0 || op == 4 || op == 7 || op == 8; }

__global__ void k_entry_count(Reads R, int64_t* cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= R.n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t n = 0;
    if (i < R.n) {
      const int64_t co = R.cigar_off[i];
      const int nc = R.n_cigar[i];
      for (int k = 0; k < nc; k++) n += entry_op((int)(R.cigar[co + k] & 15u));
    }
    cnt[i] = n;  // entry n of the array is 0: after the exclusive scan it holds the total
  }
}

__global__ void k_entry_fill(Reads R, const int64_t* off, int4* E) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < R.n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t pos = R.pos[i];
    const uint16_t fl = R.flag[i];
    const int32_t end = (fl & 0x4) ? pos : R.aend[i];
    const int32_t mq = R.mapq[i], length = R.l_seq[i];
    const int64_t co = R.cigar_off[i], qo = R.qual_off[i], so = R.seq_off[i];
    const int nc = R.n_cigar[i];
    int32_t clipped = 0;
    for (int k = 0; k < nc; k++) {
      const uint32_t w = R.cigar[co + k];
      if ((w & 15u) == 4u) clipped += (int32_t)(w >> 4);
    }
    // PileUpRegion.addRead's setup (S/PileUpRegion.scala:103-142)
    const int32_t mq1 = roundDivI(wmul(mq, length - clipped), length) + 1;
    const bool hasQual = length > 0 && R.qual[qo] != 0xFF;
    const bool pairOk = !(fl & 0x1) || ((fl & 0x2) && R.ref_id[i] == R.mate_ref_id[i]);
    const uint32_t meta = (uint32_t)mq | ((uint32_t)(fl >> 8) & 7u) << 8 | (hasQual ? kEntHasQual : 0u) |
                          (pairOk ? kEntPairOk : 0u);
    int64_t e = off[i];
    int32_t ro = 0, fo = 0;
    for (int k = 0; k < nc; k++) {
      const uint32_t w = R.cigar[co + k];
      const int32_t len = (int32_t)(w >> 4);
      const int op = (int)(w & 15u);
      const int32_t locus = pos + fo;
      if (entry_op(op)) {
        const bool clip = op == 4;
        const int32_t first = clip && ro == 0 ? locus - len : locus;  // clipStart for S
        const int64_t qa = qo + ro, na = 2 * so + ro;
        E[3 * e] = make_int4(pos, end, first, len);
        E[3 * e + 1] = make_int4(ro, length, mq1, (int32_t)(meta | (clip ? kEntClip : 0u)));
        E[3 * e + 2] = make_int4((int32_t)(uint32_t)qa, (int32_t)(qa >> 32), (int32_t)(uint32_t)na, (int32_t)(na >> 32));
        e++;
      }
      if (consumes_read(op)) ro += len;
      if (consumes_ref(op)) fo += len;
    }
  }
}

void launch_entry_count(const Reads& R, int64_t* entry_off, int64_t* sums, cudaStream_t s) {
  const int blocks = (int)std::min<int64_t>((R.n + 1 + 255) / 256, 152 * 16);
  k_entry_count<<<blocks, 256, 0, s>>>(R, entry_off);
  launch_scan64(entry_off, R.n + 1, sums, s);
}

void launch_entry_fill(const Reads& R, const int64_t* entry_off, int4* entries, cudaStream_t s) {
  if (R.n == 0) return;
  const int blocks = (int)std::min<int64_t>((R.n + 255) / 256, 152 * 16);
  k_entry_fill<<<blocks, 256, 0, s>>>(R, entry_off, entries);
}

// ---------------------------------------------------------------------------
// First index in [lo, hi) whose position is >= v (hi if none), by a warp: each
// step the 32 lanes sample the range at even strides and keep the stretch
// between the last sample below v and the next one, so a range of n reads
// takes about log32(n) steps of independent loads.
__device__ inline int64_t warp_lower_bound_pos(const int32_t* pos, int64_t lo, int64_t hi, int64_t v, int lane) {
  while (hi - lo > 32) {  // the answer lies in [lo, hi]
    const int64_t step = (hi - lo + 31) / 32;
    const int64_t sk = lo + lane * step;
    const unsigned below = __ballot_sync(FULL, sk < hi && (int64_t)pos[sk] < v);
    const int c = __popc(below);  // samples below v: lanes 0 .. c - 1
    if (c == 0) return lo;
    const int64_t nlo = lo + (int64_t)(c - 1) * step + 1;
    const int64_t sc = lo + (int64_t)c * step;
    hi = (c < 32 && sc < hi) ? sc : hi;
    lo = nlo;
  }
  const unsigned below = __ballot_sync(FULL, lo + lane < hi && (int64_t)pos[lo + lane] < v);
  return lo + __popc(below);
}

// One warp per tile.  The warp of a region's first tile also checks that the
// region's read range holds reads of the region's reference only (the range
// is searched by position, so reads of another reference would be dropped
// silently; the reference's queryOverlapping is per contig,
// S/BamFile.scala:117-119).  In a store whose references come one run each
// the first and last read decide; otherwise every read is checked.
__global__ void k_tile_ranges(Reads R, const RegionDev* regions, WalkTile* tiles, int32_t n_tiles,
                              const ReadExtent* ext, StatsDev* stats) {
  const int32_t t = (int32_t)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= n_tiles) return;  // whole warps leave together
  WalkTile& T = tiles[t];
  const RegionDev& g = regions[T.region];
  if (T.lo == 0 && g.read_end > g.read_begin) {
    bool bad = false;
    if (!ext->ungrouped) {
      bad = lane == 0 && (R.ref_id[g.read_begin] != g.contig || R.ref_id[g.read_end - 1] != g.contig);
    } else {
      for (int64_t i = g.read_begin + lane; i < g.read_end && !bad; i += 32) bad = R.ref_id[i] != g.contig;
    }
    if (__any_sync(FULL, bad) && lane == 0) stats[T.region].range_error = 1;
  }
  const int64_t tlo = (int64_t)g.start + T.lo, thi = tlo + T.len - 1;
  const int64_t a = tlo - ext->max_back, b = thi + ext->max_lead + 1;
  const int64_t rlo = warp_lower_bound_pos(R.pos, g.read_begin, g.read_end, a, lane);
  const int64_t rhi = warp_lower_bound_pos(R.pos, rlo, g.read_end, b, lane);
  if (lane == 0) {
    T.ent_lo = R.entry_off[rlo];
    T.ent_hi = R.entry_off[rhi];
  }
}

void launch_tile_ranges(const Reads& R, const RegionDev* regions, WalkTile* tiles, int32_t n_tiles,
                        const ReadExtent* ext, StatsDev* stats, cudaStream_t s) {
  if (n_tiles == 0) return;
  k_tile_ranges<<<(int)(((int64_t)n_tiles * 32 + 255) / 256), 256, 0, s>>>(R, regions, tiles, n_tiles, ext, stats);
}

// ---------------------------------------------------------------------------
// The walk kernel.  One CTA owns a tile of T positions (T a template
// parameter, so every counter address is one register plus an immediate) and
// keeps its counters in shared memory, field-major so that lanes walking
// consecutive bases of one read hit different banks:
//   md[4][T] | qx[4][T] | mx[T] | bad[T] | clips[T]     (uint32, 44 B per position)
// md[b] = sum of qual (20 bits) + count << 20 (12 bits) over the added bases b.
// M (mode_mq1) is the read store's most common adjusted mq + 1; a read whose
// mq + 1 is M + d also adds qual * d to qx[b] and d to mx.  At the flush
//   qualSum[b] = M * (sum of qual of md[b]) + qx[b]
//   mqSum      = M * (count of all four md) + mx,   qSum = sums of qual of md
// which holds for any M, so the reads of the most common mq add a base with one
// shared atomic and the others with three.  The words stay exact while a pass
// adds at most reads_per_pass reads to a position (4095: qualities are bytes,
// at most 127, so the qual sums keep within 20 bits; the API refuses a
// defaultQual outside a byte); tiles with more reads run several passes and add
// each pass's sums into the records.
//
// Each warp claims the tile's walk entries 32 at a time (one M/=/X or S
// operator of a read each, made once per read store).  Every lane reads one
// entry with three coalesced 16-byte loads and reduces it to two words and two
// addresses: the filters of BamFile.process (query window, validateRead), the
// trusted offsets of the operator inside the tile, validity and the adjusted
// mapping quality, or for an S operator its clip positions.  The warp then
// walks the lanes' entries G lanes per entry (32 / G at once), reading them by
// warp shuffle.  No CIGAR is interpreted here and no block-wide barrier runs
// inside the entry loop.
// PileUp.add of one base (S/PileUp.scala:75-84): dmq = mq + 1 - M.
template <int T>
__device__ inline void add_base(uint32_t* sm, int32_t p, uint32_t nib, int32_t qual, int32_t dmq, int32_t min_qual) {
  // nibble 1,2,4,8 (A,C,G,T) -> base index; anything else is not counted
  const uint32_t bi = (0x30210u >> (2 * nib)) & 3u;
  if (((0x116u >> nib) & 1u) && qual >= min_qual) {
    uint32_t* c = sm + p + bi * T;
    atomicAdd(c, (uint32_t)qual + (1u << 20));
    if (dmq) {
      atomicAdd(c + 4 * T, (uint32_t)(qual * dmq));
      atomicAdd(sm + 8 * T + p, (uint32_t)dmq);
    }
  }
}

// prmt.b32 in its default mode: byte k of the result is byte (s >> 4k) & 7 of
// {b:a}, or that byte's sign replicated when (s >> 4k) & 8.
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t s) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(s));
  return d;
}
// Base codes of four BAM nibbles by one prmt with the nibbles as selectors:
// A (1) -> 0x40, C (2) -> 0x41, G (4) -> 0x42 from bytes 1, 2, 4 of the table;
// T (8) -> the sign of byte 0 (0x80), 0xff; '=' (0) -> 0x80 and every other code
// -> 0x00 (bytes 3, 5-7, or the clear signs of bytes 1-7).  Bit 6 marks
// A/C/G/T and the low two bits are the base index.
constexpr uint32_t kCodeLo = 0x00414080u, kCodeHi = 0x00000042u;

__device__ inline bool nanopore_exclude(const uint8_t* cref, int32_t x, int32_t size) {
  // nanoporeExclude(index(locus)) indexes the whole contig with a region index
  return x - 2 >= 0 && x + 2 <= size - 1 && cref[x - 2] == 'C' && cref[x - 1] == 'C' && cref[x + 1] == 'G' &&
         cref[x + 2] == 'G';
}

// PileUp.add (S/PileUp.scala:75-84) of the four bases of one chunk: qv holds
// their quality bytes, sv their nibbles from the chunk's first byte on (see
// comb in the walk).  The nibbles select their codes (kCodeLo/Hi) by prmt; a
// second prmt puts code j in byte j.  DMQ: the entry's mq + 1 differs from the
// store's most common value, so qual * dmq and dmq go to the correction words.
template <int T, bool DMQ>
__device__ __forceinline__ void add_chunk(uint32_t* cl, uint32_t qv, uint32_t sv, uint32_t comb, uint32_t minq4,
                                          uint32_t okall, int32_t dmq) {
  const uint32_t code = prmt(prmt(kCodeLo, kCodeHi, sv), prmt(kCodeLo, kCodeHi, sv >> 8), comb);
  // bit 6 of byte j: base j is A/C/G/T and its quality byte is in [minQual, 127]
  const uint32_t ok = code & ((((qv | 0x80808080u) - minq4) & ~qv & 0x80808080u) >> 1) & okall;
  const uint32_t qm = qv & ((ok >> 6) * 0x7fu);  // accepted qualities, 0 elsewhere
  const uint32_t one4 = ok >> 2;                 // 0x10 in the bytes of accepted bases
  const uint32_t bix = code & 0x03030303u;       // base index of byte j (0 when rejected)
  // base j adds qual + (1 << 20), built by one prmt: byte 0 = quality, byte 2 =
  // 0x10 or 0, bytes 1 and 3 = the clear sign of a byte of one4; a rejected base
  // adds 0 to row 0 (no branch per base)
#pragma unroll
  for (int j = 0; j < 4; j++)
    atomicAdd(cl + j + prmt(bix, 0u, 0x4440u | (uint32_t)j) * T,
              prmt(qm, one4, (uint32_t)(j | (12 + j) << 4 | (4 + j) << 8 | (12 + j) << 12)));
  if (DMQ) {  // qual * dmq to qx[b], dmq to mx (0 for a rejected base)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      atomicAdd(cl + 4 * T + j + prmt(bix, 0u, 0x4440u | (uint32_t)j) * T,
                prmt(qm, 0u, 0x4440u | (uint32_t)j) * (uint32_t)dmq);
      atomicAdd(cl + 8 * T + j, ((ok >> (8 * j + 6)) & 1u) * (uint32_t)dmq);
    }
  }
}

// The whole chunks c = c0, c0 + G, ... < cend of one entry for one lane: chunk
// c's qualities are word c of qw, its nibbles start at byte sb + 2c of the
// sequence (every such byte sits at the same offset in its aligned word, so two
// aligned words and a funnel shift give them).  Two chunks are added per
// iteration while the next two load.
template <int T, int G, bool DMQ>
__device__ __forceinline__ void walk_chunks(uint32_t* cbase, const uint32_t* qw, const uint8_t* seq, int64_t sb,
                                            int32_t c0, int32_t cend, uint32_t lastb, uint32_t comb, uint32_t minq4,
                                            uint32_t okall, int32_t dmq) {
  if (c0 >= cend) return;
  const uintptr_t ba0 = (uintptr_t)(seq + sb + 2 * c0);
  const uint32_t sh = 8u * (uint32_t)(ba0 & 3u);
  const bool need_hi = (ba0 & 3u) + lastb >= 4u;
  const uint32_t* wp = (const uint32_t*)(ba0 & ~(uintptr_t)3);  // word of chunk c0; chunk c0 + kG at wp + k G / 2
  auto load = [&](int32_t k, uint32_t& q, uint32_t& sv) {  // the lane's k-th chunk
    const uint32_t* w = wp + k * (G / 2);
    const uint32_t lo = w[0], hi = need_hi ? w[1] : 0u;
    q = qw[c0 + k * G];
    sv = __funnelshift_r(lo, hi, sh);
  };
  const int32_t n = (cend - c0 + G - 1) / G;  // chunks of this lane
  uint32_t qa = 0, sa = 0, qb = 0, sb2 = 0;
  load(0, qa, sa);
  if (n > 1) load(1, qb, sb2);
  for (int32_t k = 0; k < n; k += 2) {
    uint32_t qc = 0, sc = 0, qd = 0, sd = 0;
    if (k + 2 < n) load(k + 2, qc, sc);
    if (k + 3 < n) load(k + 3, qd, sd);
    add_chunk<T, DMQ>(cbase + 4 * (c0 + k * G), qa, sa, comb, minq4, okall, dmq);
    if (k + 1 < n) add_chunk<T, DMQ>(cbase + 4 * (c0 + (k + 1) * G), qb, sb2, comb, minq4, okall, dmq);
    qa = qc; sa = sc; qb = qd; sb2 = sd;
  }
}

// entry kinds of a lane's word w1
enum : uint32_t { kSkip = 0, kFast = 1, kInvalid = 2, kSlow = 3, kClip = 4 };

// dynamic shared memory of a walk CTA: the counters and 4 words of padding
template <int T>
constexpr size_t walk_smem() {
  return (size_t)(11 * T + 4) * sizeof(uint32_t);
}

// MINB: resident CTAs the register allocation must allow: 2 CTAs of up to 512
// threads (16 warps, up to 64 registers per thread) or 5 CTAs of up to 256
// threads (8 warps, up to 48 registers: 40 warps per SM).  G: lanes per entry
// (4, 8, 16, 32).
template <int T, int MINB, int G>
__global__ void __launch_bounds__(MINB >= 4 ? 256 : 512, MINB) k_walk(WalkArgs a, int32_t tile_begin,
                                                                      int32_t tile_end) {
  constexpr int kWords = 11 * T;
  static_assert((kWords + 4) % 4 == 0, "counters are cleared 16 bytes at a time");
  extern __shared__ __align__(16) uint32_t sm_raw[];
  uint32_t* sm = sm_raw + 4;  // 4 words of padding in front of the counters
  __shared__ unsigned long long s_bc;
  __shared__ uint8_t s_perm[16][32];  // per warp: lane of the entry in each round slot
  __shared__ int32_t s_next;          // next unclaimed entry of the pass (offset)
  uint32_t* s_bad = sm + 9 * T;  // md = sm, qx = sm + 4T, mx = sm + 8T
  uint32_t* s_clip = sm + 10 * T;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int gl = lane % G, grp = lane / G;
  constexpr int NG = 32 / G;
  const Reads& R = a.R;
  const DevParams& P = a.P;
  const uint32_t mode_mq1 = a.mode_mq1;
  // minQual in every byte: ((q | 0x80) - minQual) keeps bit 7 iff q >= minQual,
  // for q < 128; no quality byte passes a minQual above 127
  const uint32_t minq4 = (uint32_t)min(max(P.min_qual, 0), 127) * 0x01010101u;
  const uint32_t okall = P.min_qual <= 127 ? 0xffffffffu : 0u;
  const int64_t per_pass = a.reads_per_pass;
  // validateRead (S/BamFile.scala:101-105) on the entry's flag bits 0x100
  // (always dropped), 0x200 (unless --nonpf) and 0x400 (unless --duplicates)
  const uint32_t drop = (1u | (P.nonpf ? 0u : 2u) | (P.duplicates ? 0u : 4u)) << 8;
  const bool nanopore = P.long_read == PG_NANOPORE;
  const int4* __restrict__ ent = R.entries;

  for (int32_t t = tile_begin + blockIdx.x; t < tile_end; t += gridDim.x) {
    const WalkTile tile = a.tiles[t];
    const RegionDev g = a.regions[tile.region];
    const int32_t tileLo = g.start + tile.lo, tileHi = tileLo + tile.len - 1;
    const uint8_t* cref = a.ref + g.ref_off;
    unsigned long long bc = 0;
    if (threadIdx.x == 0) s_bc = 0;

    for (int64_t c0 = tile.ent_lo, pass = 0; pass == 0 || c0 < tile.ent_hi; c0 += per_pass, pass++) {
      const int64_t c1 = min(c0 + per_pass, tile.ent_hi);
      const int32_t npass = (int32_t)(c1 - c0);
      for (int k = threadIdx.x; k < (kWords + 4) / 4; k += blockDim.x)
        reinterpret_cast<uint4*>(sm_raw)[k] = make_uint4(0u, 0u, 0u, 0u);
      if (threadIdx.x == 0) s_next = 0;
      __syncthreads();

      // Warps claim batches of the pass's entries as they finish the previous
      // one: 32 while many are left, then 16, then 8, so the warps reach the
      // tile's closing barrier close together.
      while (true) {
        int32_t off = 0, size = 0;
        if (lane == 0) {
          const int32_t rem = npass - *(volatile int32_t*)&s_next;
          size = rem > 64 * nwarps ? 32 : rem > 16 * nwarps ? 16 : 8;
          off = atomicAdd(&s_next, size);
        }
        off = __shfl_sync(FULL, off, 0);
        size = __shfl_sync(FULL, size, 0);
        if (off >= npass) break;
        const int64_t base = c0 + off, bend = min(base + size, c1);
        // ---- one entry per lane, reduced to w0 = first tile position | count << 16,
        // w1 = kind | flags | (adjMq + 1 or clip positions) << 8, and the quality
        // byte and nibble index of the first base
        const int64_t k = base + lane;
        uint32_t w0 = 0, w1 = kSkip;
        uint64_t qa = 0, na = 0;
        int32_t cls = 0;
        if (k < bend) {
          const int4 e0 = __ldg(ent + 3 * k), e1 = __ldg(ent + 3 * k + 1), e2 = __ldg(ent + 3 * k + 2);
          const uint32_t meta = (uint32_t)e1.w;
          if (e0.x <= g.qe && e0.y >= g.qs && !(meta & drop)) {
            const int32_t first = e0.z, len = e0.w;
            if (meta & kEntClip) {
              // S (S/PileUpRegion.scala:194-206): clips at clipStart and clipEnd, and
              // every clipped base is added as a bad pair, for valid and invalid reads
              const int32_t ce = first + len - 1;
              const int32_t lo = max(first, tileLo), hi = min(ce, tileHi);
              const bool csin = first >= tileLo && first <= tileHi, cein = ce >= tileLo && ce <= tileHi;
              if (lo <= hi || csin || cein) {
                w0 = lo <= hi ? (uint32_t)(lo - tileLo) | (uint32_t)(hi - lo + 1) << 16 : 0u;
                w1 = kClip | (csin ? 8u : 0u) | (cein ? 16u : 0u) | ((uint32_t)(first - tileLo) & 0xfffu) << 8 |
                     ((uint32_t)(ce - tileLo) & 0xfffu) << 20;
              }
            } else {
              // M/=/X (S/PileUpRegion.scala:184-193): the trusted read offsets
              // [flank, length - flank) of the operator, inside the tile
              const int32_t roff = e1.x, rlen = e1.y, mq1 = e1.z;
              const int32_t i0 = max(max(tileLo - first, P.flank - roff), 0);
              const int32_t i1 = min(min(tileHi - first + 1, rlen - P.flank - roff), len);
              if (i1 > i0) {
                const bool valid = (int32_t)(meta & 0xffu) >= P.min_mq && (meta & kEntPairOk);
                const bool hasQual = (meta & kEntHasQual) != 0;
                if (valid) bc += (unsigned long long)(i1 - i0);
                const uint32_t kind =
                    !valid ? kInvalid : (hasQual && !nanopore && mq1 >= 1 && mq1 <= 256) ? kFast : kSlow;
                const int32_t pb = first + i0 - tileLo;
                w0 = (uint32_t)pb | (uint32_t)(i1 - i0) << 16;
                w1 = kind | (hasQual ? 8u : 0u) | (uint32_t)mq1 << 8;
                qa = ((uint64_t)(uint32_t)e2.y << 32 | (uint32_t)e2.x) + (uint64_t)i0;
                na = ((uint64_t)(uint32_t)e2.w << 32 | (uint32_t)e2.z) + (uint64_t)i0;
                // position residue (mod 4) of the entry's 4-base chunks, which start
                // at the aligned quality words (see the fast path)
                cls = (pb - (int32_t)((uintptr_t)(R.qual + qa) & 3u)) & 3;
              }
            }
          }
        }
        // ---- the lanes' entries, NG at a time, G lanes each.  With 4 groups, round k
        // gives group g the k-th entry of residue class g while every class has one,
        // so the groups add to 4 different position residues at every step and their
        // shared-memory atomics hit 32 different banks; the entries left over follow
        // in lane order.  Each lane computes its entry's slot at once.
        const uint32_t kind = w1 & 7u;
        const unsigned below = (1u << lane) - 1u;
        const unsigned act_all = __ballot_sync(FULL, kind != kSkip);
        const int n_act = __popc(act_all);
        if (kind != kSkip) {
          // entries of the most common mq first (so that rounds mix one-atomic and
          // three-atomic adds at most once), interleaved by residue class; the rest after
          const bool first = kind == kFast && (uint32_t)((int32_t)w1 >> 8) == mode_mq1;
          const unsigned set_a = __ballot_sync(act_all, first);
          int slot;
          if (first) {
            if (NG == 4 || NG == 8) {  // with 8 groups, groups g and g + 4 share a residue class
              const unsigned c0m = __ballot_sync(set_a, cls == 0), c1m = __ballot_sync(set_a, cls == 1);
              const unsigned c2m = __ballot_sync(set_a, cls == 2), c3m = __ballot_sync(set_a, cls == 3);
              const int m = min(min(__popc(c0m), __popc(c1m)), min(__popc(c2m), __popc(c3m)));
              const unsigned mine = cls == 0 ? c0m : cls == 1 ? c1m : cls == 2 ? c2m : c3m;
              const int rank = __popc(mine & below);
              const unsigned left = __ballot_sync(set_a, rank >= m);
              slot = rank < m ? 4 * rank + cls : 4 * m + __popc(left & below);
            } else {
              slot = __popc(set_a & below);
            }
          } else {
            slot = __popc(set_a) + __popc(act_all & ~set_a & below);
          }
          s_perm[warp][slot] = (uint8_t)lane;
        }
        __syncwarp();
        for (int r0 = 0; r0 < n_act; r0 += NG) {
          const int src = r0 + grp < n_act ? (int)s_perm[warp][r0 + grp] : 32;  // 32: no entry for this group
          const int s2 = src < 32 ? src : lane;
          const uint32_t rw0 = __shfl_sync(FULL, w0, s2), rw1 = __shfl_sync(FULL, w1, s2);
          const uint64_t rqa = __shfl_sync(FULL, qa, s2), rna = __shfl_sync(FULL, na, s2);
          if (src < 32) {
            const uint32_t rk = rw1 & 7u;
            const int32_t rpb = (int32_t)(rw0 & 0xffffu), rn = (int32_t)(rw0 >> 16);
            if (rk == kFast) {
              // Whole chunks of 4 consecutive bases that start on an aligned quality
              // word; lane gl of the group takes chunks cf + gl, cf + gl + G, ...
              // (walk_chunks: two added while the next two load).  A chunk's qualities
              // are one aligned word and its nibbles lie in at most two aligned
              // sequence words, each holding one of the entry's bytes, so no load
              // leaves the pages of the read store.  The at most 6 bases before the
              // first and after the last whole chunk are added one per lane.
              const uint8_t* rqp = R.qual + rqa;  // quality of base 0 (tile position rpb)
              const uintptr_t qaddr = (uintptr_t)rqp;
              const int32_t e0 = (int32_t)(qaddr & 3u);
              const int32_t xs = -e0;  // base index of byte 0 of chunk 0
              const uint32_t* qw = (const uint32_t*)(qaddr - (uintptr_t)e0);
              const int32_t cf = e0 ? 1 : 0, cend = (rn - xs) >> 2;  // whole chunks [cf, cend)
              const int32_t fs = xs + 4 * cf, fe = xs + 4 * max(cend, cf);
              const int32_t he = min(fs, rn), ts = max(fe, he), nh = he, nt = max(rn - ts, 0);
              // head and tail bases: loaded now, added after the chunks
              constexpr int kHT = (6 + G - 1) / G;  // head/tail bases per lane
              int32_t hx[kHT];
              uint32_t hb[kHT], hq[kHT];
#pragma unroll
              for (int h = 0; h < kHT; h++) {
                const int32_t kk = gl + h * G;
                hx[h] = kk < nh + nt ? (kk < nh ? kk : ts + (kk - nh)) : -1;
                hb[h] = hq[h] = 0;
                if (hx[h] >= 0) {
                  hb[h] = R.seq[(rna + (uint64_t)hx[h]) >> 1];
                  hq[h] = rqp[hx[h]];
                }
              }
              const int64_t n0 = (int64_t)rna + xs;  // nibble index of chunk 0's first base
              const uint32_t lastb = (uint32_t)((n0 & 1) + 3) >> 1;  // last byte of a chunk's nibbles
              // sv holds a chunk's nibbles from its first byte on: with an even nibble
              // index bases 1, 0, 3, 2 in its low four nibbles; with an odd one bases 0
              // and 2 in nibbles 0 and 2, base 1 in nibble 3 and base 3 in nibble 5
              const uint32_t comb = (n0 & 1) ? 0x7230u : 0x2301u;
              // mq + 1 - M: 0 for the entries of the most common mq
              const int32_t dmq = ((int32_t)rw1 >> 8) - (int32_t)mode_mq1;
              // chunk c's counters start at tile position rpb + xs + 4c; its first
              // nibble is in byte (n0 >> 1) + 2c (chunk 0 is used only when n0 >= 0)
              uint32_t* cbase = sm + (rpb + xs);
              if (dmq == 0)
                walk_chunks<T, G, false>(cbase, qw, R.seq, n0 >> 1, cf + gl, cend, lastb, comb, minq4, okall, 0);
              else
                walk_chunks<T, G, true>(cbase, qw, R.seq, n0 >> 1, cf + gl, cend, lastb, comb, minq4, okall, dmq);
#pragma unroll
              for (int h = 0; h < kHT; h++) {
                if (hx[h] < 0) continue;
                const uint32_t nib = ((rna + (uint64_t)hx[h]) & 1u) ? (hb[h] & 15u) : (hb[h] >> 4);
                add_base<T>(sm, rpb + hx[h], nib, (int32_t)(int8_t)hq[h], dmq, P.min_qual);
              }
            } else if (rk == kInvalid) {  // add() of an invalid read: badPair (S/PileUpRegion.scala:38-48)
              for (int32_t ii = gl; ii < rn; ii += G) atomicAdd(&s_bad[rpb + ii], 1u);
            } else if (rk == kSlow) {  // no qualities (defaultQual), nanopore motifs, or an mq outside a byte
              const bool rhas = (rw1 & 8u) != 0;
              const int32_t dmq = ((int32_t)rw1 >> 8) - (int32_t)mode_mq1;
              for (int32_t ii = gl; ii < rn; ii += G) {
                const uint64_t ni = rna + (uint64_t)ii;
                const uint8_t b = R.seq[ni >> 1];
                const uint32_t nib = (ni & 1u) ? (b & 15u) : (uint32_t)(b >> 4);
                int32_t qual = rhas ? (int32_t)(int8_t)R.qual[rqa + (uint64_t)ii] : P.default_qual;
                if (nanopore && nanopore_exclude(cref, tileLo + rpb + ii - g.start, g.size)) qual = 0;
                add_base<T>(sm, rpb + ii, nib, qual, dmq, P.min_qual);
              }
            } else {  // kClip
              if (gl == 0) {
                if (rw1 & 8u) atomicAdd(&s_clip[(rw1 >> 8) & 0xfffu], 1u);
                if (rw1 & 16u) atomicAdd(&s_clip[rw1 >> 20], 1u);
              }
              for (int32_t ii = gl; ii < rn; ii += G) atomicAdd(&s_bad[rpb + ii], 1u);
            }
          }
        }
        __syncwarp();
      }
      __syncthreads();

      // flush: the first pass stores, later passes add (the CTA owns the tile)
      for (int32_t p = threadIdx.x; p < tile.len; p += blockDim.x) {
        const int64_t gp = g.pos_base + tile.lo + p;
        const uint32_t M = mode_mq1;
        const uint32_t w0 = sm[p], w1 = sm[T + p], w2 = sm[2 * T + p], w3 = sm[3 * T + p];
        const int4 c = make_int4((int)(w0 >> 20), (int)(w1 >> 20), (int)(w2 >> 20), (int)(w3 >> 20));
        const uint32_t s0 = w0 & 0xFFFFFu, s1 = w1 & 0xFFFFFu, s2 = w2 & 0xFFFFFu, s3 = w3 & 0xFFFFFu;
        // qx and mx hold signed per-pass sums within int32
        const longlong2 q01 = make_longlong2((long long)M * s0 + (int32_t)sm[4 * T + p],
                                             (long long)M * s1 + (int32_t)sm[5 * T + p]);
        const longlong2 q23 = make_longlong2((long long)M * s2 + (int32_t)sm[6 * T + p],
                                             (long long)M * s3 + (int32_t)sm[7 * T + p]);
        const int32_t mqs = wadd((int32_t)(M * (uint32_t)(c.x + c.y + c.z + c.w)), (int32_t)sm[8 * T + p]);
        const int32_t qsum = (int32_t)(s0 + s1 + s2 + s3);
        if (pass == 0) {
          a.rec.count[gp] = c;
          a.rec.qual_sum[2 * gp] = q01;
          a.rec.qual_sum[2 * gp + 1] = q23;
          a.rec.mq_sum[gp] = mqs;
          a.rec.q_sum[gp] = qsum;
          a.rec.bad_pair[gp] = (int32_t)s_bad[p];
          a.rec.clips[gp] = (int32_t)s_clip[p];
          a.rec.deletions[gp] = 0;
          a.rec.del_qual[gp] = 0;
          a.rec.insertions[gp] = 0;
          a.rec.ins_qual[gp] = 0;
          a.rec.phys_cov[gp] = 0;
          a.rec.insert_size[gp] = 0;
        } else {
          const int4 o = a.rec.count[gp];
          a.rec.count[gp] = make_int4(o.x + c.x, o.y + c.y, o.z + c.z, o.w + c.w);
          const longlong2 o1 = a.rec.qual_sum[2 * gp], o2 = a.rec.qual_sum[2 * gp + 1];
          a.rec.qual_sum[2 * gp] = make_longlong2(o1.x + q01.x, o1.y + q01.y);
          a.rec.qual_sum[2 * gp + 1] = make_longlong2(o2.x + q23.x, o2.y + q23.y);
          a.rec.mq_sum[gp] = wadd(a.rec.mq_sum[gp], mqs);
          a.rec.q_sum[gp] = wadd(a.rec.q_sum[gp], qsum);
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

template <int T, int MINB, int G>
static void launch_walk_t(const WalkArgs& a, int32_t tile_begin, int32_t tile_count, int warps, cudaStream_t s) {
  const size_t smem = walk_smem<T>();
  // attribute and occupancy are queried once per (kernel, warps): the first
  // launch of a shape is never inside a stream capture
  static bool configured = false;
  static int per_sm_of[17] = {0};
  if (!configured) {
    cudaFuncSetAttribute(k_walk<T, MINB, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = true;
  }
  if (!per_sm_of[warps]) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk<T, MINB, G>, warps * 32, smem);
    per_sm_of[warps] = std::max(per_sm, 1);
  }
  const int per_sm = per_sm_of[warps];
  const int blocks = std::min(tile_count, 152 * per_sm);
  k_walk<T, MINB, G><<<blocks, warps * 32, smem, s>>>(a, tile_begin, tile_begin + tile_count);
}

template <int MINB, int G>
static void launch_walk_v(const WalkArgs& a, int32_t tile_begin, int32_t tile_count, int warps, cudaStream_t s) {
  switch (a.tile_width) {
    case 256: launch_walk_t<256, MINB, G>(a, tile_begin, tile_count, warps, s); break;
    case 512: launch_walk_t<512, MINB, G>(a, tile_begin, tile_count, warps, s); break;
    case 1024: launch_walk_t<1024, MINB, G>(a, tile_begin, tile_count, warps, s); break;
    case 2048: launch_walk_t<2048, MINB, G>(a, tile_begin, tile_count, warps, s); break;
    default: launch_walk_t<4096, MINB, G>(a, tile_begin, tile_count, warps, s); break;
  }
}

// variant: lanes per simple read (0: 32, 1: 16, 2: 8, 3: 4).
void launch_walk(const WalkArgs& a, int32_t tile_begin, int32_t tile_count, int warps, cudaStream_t s) {
  if (tile_count <= 0) return;
  const int lanes = a.packed;
  if (warps <= 8) {  // 256-thread CTAs, 5 resident per SM
    if (lanes == 0) launch_walk_v<5, 32>(a, tile_begin, tile_count, warps, s);
    else if (lanes == 1) launch_walk_v<5, 16>(a, tile_begin, tile_count, warps, s);
    else if (lanes == 2) launch_walk_v<5, 8>(a, tile_begin, tile_count, warps, s);
    else launch_walk_v<5, 4>(a, tile_begin, tile_count, warps, s);
  } else {
    if (lanes == 0) launch_walk_v<2, 32>(a, tile_begin, tile_count, warps, s);
    else if (lanes == 1) launch_walk_v<2, 16>(a, tile_begin, tile_count, warps, s);
    else if (lanes == 2) launch_walk_v<2, 8>(a, tile_begin, tile_count, warps, s);
    else launch_walk_v<2, 4>(a, tile_begin, tile_count, warps, s);
  }
}

// ---------------------------------------------------------------------------
// Per (region, read): readCount, insert statistics, physCovIncr and indels.
__device__ inline unsigned long long warp_sum_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
  return v;
}

// kEvThreads threads per CTA, kReadsPerChunk / kEvThreads CTAs per read chunk,
// one read per thread.  Each warp adds its partial sums into the chunk's
// (zeroed) statistics with global atomics, so no warp waits for another: the
// few reads with indels run long left-shift loops.
constexpr int kEvThreads = 64;
constexpr int kEvPerChunk = kReadsPerChunk / kEvThreads;
static_assert(kEvPerChunk * kEvThreads == kReadsPerChunk, "one read per thread of k_read_events");

__global__ void __launch_bounds__(kEvThreads, 20) k_read_events(EventArgs a, int32_t chunk_begin, int32_t chunk_end) {
  const Reads& R = a.R;
  const DevParams& P = a.P;
  for (int32_t bq = chunk_begin * kEvPerChunk + blockIdx.x; bq < chunk_end * kEvPerChunk; bq += gridDim.x) {
    const int32_t ch = bq / kEvPerChunk;
    const ReadChunk C = a.chunks[ch];
    const RegionDev g = a.regions[C.region];
    unsigned long long rc_n = 0, bc_n = 0, frc = 0, frs = 0, frq = 0, rfc = 0, rfs = 0, rfq = 0;
    uint32_t pcs = 0, iss = 0;
    int32_t err = 0;
    int64_t indel_read = -1;  // this thread's read, when it has I or D operators
    auto inRegion = [&](int64_t l) { return l >= g.start && l <= g.stop; };
    for (int64_t i = C.lo + (int64_t)(bq % kEvPerChunk) * kEvThreads + threadIdx.x; i < C.hi;
         i += (int64_t)kEvPerChunk * kEvThreads) {
      // all loads of a read are independent: the per-store descriptor holds the CIGAR shape
      const int4 d0 = R.desc[2 * i], d1 = R.desc[2 * i + 1];
      const int32_t aend = R.aend[i], tlen = R.tlen[i];
      const uint16_t fl = R.flag[i];
      const int32_t mq = R.mapq[i];
      const int32_t pos = d0.x;
      if (d0.z != g.contig || !(pos <= g.qe && d0.y >= g.qs) || !validate_read(fl, P)) continue;
      rc_n++;
      const bool paired = fl & 0x1;
      const bool valid = (mq >= P.min_mq) && ((uint32_t)d1.z & kDescPairOk);

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
          pcs += 1u;
          iss += (uint32_t)insertSize;
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
        if (fr) { frc++; frs += (unsigned long long)insertSize; frq += sq; }
        else { rfc++; rfs += (unsigned long long)insertSize; rfq += sq; }
      }

      // reads with I or D operators go to k_read_indels
      if (valid && !((uint32_t)d1.y & kDescSimple) && d1.x != 0) indel_read = i;
    }
    {  // list them in the chunk's slots: one atomic per warp on the chunk's counter
      const unsigned m = __ballot_sync(FULL, indel_read >= 0);
      if (m) {
        const int lane = threadIdx.x & 31;
        int32_t first = 0;
        if (lane == __ffs(m) - 1) first = atomicAdd(&a.chunk_stats[ch].n_indel, __popc(m));
        first = __shfl_sync(FULL, first, __ffs(m) - 1);
        if (indel_read >= 0)
          a.indel_list[(int64_t)ch * kReadsPerChunk + first + __popc(m & ((1u << lane) - 1u))] = indel_read;
      }
    }
    rc_n = warp_sum_u64(rc_n); bc_n = warp_sum_u64(bc_n);
    frc = warp_sum_u64(frc); frs = warp_sum_u64(frs); frq = warp_sum_u64(frq);
    rfc = warp_sum_u64(rfc); rfs = warp_sum_u64(rfs); rfq = warp_sum_u64(rfq);
    pcs = __reduce_add_sync(FULL, pcs); iss = __reduce_add_sync(FULL, iss);
    err = __reduce_max_sync(FULL, err);
    if ((threadIdx.x & 31) == 0) {  // k_region_prep adds the chunks up per region
      ChunkStats& cs = a.chunk_stats[ch];
      if (rc_n) atomicAdd(&cs.read_count, rc_n);
      if (bc_n) atomicAdd(&cs.base_count, bc_n);
      if (frc) { atomicAdd(&cs.fr_count, frc); atomicAdd(&cs.fr_sum, frs); atomicAdd(&cs.fr_sumsq, frq); }
      if (rfc) { atomicAdd(&cs.rf_count, rfc); atomicAdd(&cs.rf_sum, rfs); atomicAdd(&cs.rf_sumsq, rfq); }
      if (pcs) atomicAdd((uint32_t*)&cs.phys_cov_start, pcs);
      if (iss) atomicAdd((uint32_t*)&cs.insert_size_start, iss);
      if (err) atomicMax(&cs.error, err);
    }
  }
}

// The I and D operators of the listed reads (S/PileUpRegion.scala:150-183):
// left shift, H1 double count, the indel counters and the events for the
// vote.  Each warp takes the lists of kIndelChunks chunks (a few per cent of
// their reads have indels) and walks their union 32 reads at a time, one
// read per thread: the in-warp scan of the lists' lengths gives each entry's
// list, as the last list starting at or before it.
constexpr int kIndelThreads = 128, kIndelChunks = 2;
__global__ void __launch_bounds__(kIndelThreads) k_read_indels(EventArgs a, int32_t chunk_begin, int32_t chunk_end) {
  __shared__ uint8_t s_lane[kIndelThreads / 32][32];  // per warp: lane of the k-th non-empty list
  const Reads& R = a.R;
  const DevParams& P = a.P;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int32_t c0 = chunk_begin + (int32_t)(((int64_t)blockIdx.x * kIndelThreads + threadIdx.x) >> 5) * kIndelChunks;
  if (c0 >= chunk_end) return;  // whole warps leave together
  const int32_t cnt = (lane < kIndelChunks && c0 + lane < chunk_end) ? a.chunk_stats[c0 + lane].n_indel : 0;
  int32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t v = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += v;
  }
  const int32_t E = incl - cnt, total = __shfl_sync(FULL, incl, 31);
  const unsigned ne = __ballot_sync(FULL, cnt > 0);
  if (cnt > 0) s_lane[wib][__popc(ne & ((1u << lane) - 1u))] = (uint8_t)lane;
  __syncwarp();
  for (int32_t k0 = 0; k0 < total; k0 += 32) {
    // the non-empty list holding entry k0, then one more per list start in (k0, k0 + lane]
    const int r0 = __popc(__ballot_sync(FULL, cnt > 0 && E <= k0)) - 1;
    const uint32_t st = (cnt > 0 && E > k0 && E < k0 + 32) ? 1u << (E - k0) : 0u;
    const int rk = r0 + __popc(__reduce_or_sync(FULL, st) & ((2u << lane) - 1u));
    const int own = k0 + lane < total ? (int)s_lane[wib][rk] : lane;
    const int32_t ownE = __shfl_sync(FULL, E, own);
    const int32_t ch = c0 + own;
    int64_t i = -1;
    int32_t n_id = 0;  // I and D operators of the read: one event slot each
    if (k0 + lane < total) {
      i = a.indel_list[(int64_t)ch * kReadsPerChunk + (k0 + lane - ownE)];
      const int64_t co = R.cigar_off[i];
      const int nc = R.n_cigar[i];
      for (int k = 0; k < nc; k++) {
        const uint32_t op = R.cigar[co + k] & 15u;
        n_id += (op == 1u || op == 2u);
      }
    }
    // the warp's event slots, reserved with one atomic; an operator that adds
    // no event leaves its slot empty (gpos -1), which k_event_scatter skips
    int32_t ev_incl = n_id;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t v = __shfl_up_sync(FULL, ev_incl, o);
      if (lane >= o) ev_incl += v;
    }
    unsigned long long ev_base = 0;
    if (lane == 31 && ev_incl > 0) ev_base = atomicAdd(a.n_events, (unsigned long long)ev_incl);
    ev_base = __shfl_sync(FULL, ev_base, 31);
    if (i < 0) continue;
    unsigned long long ev_next = ev_base + (unsigned long long)(ev_incl - n_id);
    const ReadChunk C = a.chunks[ch];
    const RegionDev g = a.regions[C.region];
    const uint8_t* cref = a.ref + g.ref_off;
    auto inRegion = [&](int64_t l) { return l >= g.start && l <= g.stop; };
    const int4 d0 = R.desc[2 * i], d1 = R.desc[2 * i + 1];
    const int32_t pos = d0.x;
    unsigned long long bc_n = 0;
    int32_t err = 0;
    {
      const int64_t co = R.cigar_off[i];
      const int nc = R.n_cigar[i];
      const int32_t length = R.l_seq[i];
      const uint8_t* rseq = R.seq + R.seq_off[i];   // loaded once per read
      const uint8_t* rqual = R.qual + R.qual_off[i];
      auto nib = [&](int32_t k) -> uint32_t {
        const uint8_t b = rseq[k >> 1];
        return (k & 1) ? (b & 15u) : (uint32_t)(b >> 4);
      };
      const int32_t adjMq = d0.w - 1;
      const int32_t indelMq = P.long_read > 0 ? min(adjMq, 8) : adjMq;
      const bool hasQual = ((uint32_t)d1.y & kDescHasQual) != 0;
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
        const unsigned long long my_slot = (op == 1 || op == 2) ? ev_next++ : 0ull;
        bool wrote = false;
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
            if (rb != nib_char(nib(readOffset + kk))) break;
            iloc -= 1;
            rot += 1;
            if (rot == len) rot = 0;
          }
          if (!bad && P.long_read > 0) {
            if (homoRun(iloc, bad) >= 4 && !bad) goto next_op;
          }
          if (bad || iloc < g.start) { err = PG_ERR_INDEX; goto next_op; }
          {
            const int64_t gp = g.pos_base + (iloc - g.start);
            atomicAdd(&a.rec.ins_qual[gp], indelMq + 1);
            atomicAdd(&a.rec.q_sum[gp], (hasQual ? (int32_t)(int8_t)rqual[readOffset] : P.default_qual));
            atomicAdd(&a.rec.insertions[gp], 1);
            const unsigned long long slot = my_slot;
            wrote = true;
            if ((int64_t)slot < a.event_cap) {
              Event e;
              e.gpos = gp; e.read = i; e.region = C.region; e.len = len; e.roff = readOffset; e.kind_rot = rot;
              // the rotated string as 4-bit codes: characters 0..15 in the key,
              // the rest 16 per word in the string pool
              uint64_t key = 0;
              for (int32_t j = 0; j < min(len, 16); j++) {
                int32_t kk = j - rot;
                if (kk < 0) kk += len;
                key |= (uint64_t)nib(readOffset + kk) << (60 - 4 * j);
              }
              e.key = key;
              e.sp = -1;
              if (len > 16) {
                const int32_t nw = (len - 16 + 15) / 16;
                const unsigned long long sp = atomicAdd(a.spool_fill, (unsigned long long)nw);
                if ((int64_t)(sp + nw) <= a.spool_cap) {
                  for (int32_t w = 0; w < nw; w++) {
                    uint64_t word = 0;
                    for (int32_t j = 16 + 16 * w; j < min(len, 32 + 16 * w); j++) {
                      int32_t kk = j - rot;
                      if (kk < 0) kk += len;
                      word |= (uint64_t)nib(readOffset + kk) << (60 - 4 * (j - 16 - 16 * w));
                    }
                    a.spool[sp + w] = word;
                  }
                  e.sp = (int64_t)sp;
                } else {
                  e.len = -1;  // pool full: the host grows it and runs again
                }
              }
              a.events[slot] = e;
            }
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
                const int bi = nib_index(nib(rloc));
                const int32_t q = (hasQual ? (int32_t)(int8_t)rqual[rloc] : P.default_qual);
                if (bi >= 0 && q >= P.min_qual) {
                  atomicAdd(((int*)a.rec.count) + 4 * gp + bi, 1);
                  atomicAdd(((unsigned long long*)a.rec.qual_sum) + 4 * gp + bi,
                            (unsigned long long)(long long)wmul(q, adjMq + 1));
                  atomicAdd(&a.rec.mq_sum[gp], adjMq + 1);
                  atomicAdd(&a.rec.q_sum[gp], q);
                }
                bc_n++;
              }
            }
          }
          if (bad) { err = PG_ERR_INDEX; goto next_op; }
          if (P.long_read > 0) {
            const int64_t i0 = (int64_t)dloc - g.start;  // index(dloc), used as a contig index
            if (homoRun(i0, bad) >= 4 && !bad) goto next_op;
            if (!bad && P.long_read == PG_NANOPORE) {
              bool ex = (i0 - 2 >= 0) && (i0 + 2 <= g.size - 1) && cref[i0 - 2] == 'C' && cref[i0 - 1] == 'C' &&
                        cref[i0 + 1] == 'G' && cref[i0 + 2] == 'G';
              if (ex) goto next_op;
            }
          }
          if (bad || dloc < g.start) { err = PG_ERR_INDEX; goto next_op; }
          {
            const int64_t gp = g.pos_base + (dloc - g.start);
            atomicAdd(&a.rec.mq_sum[gp], indelMq + 1);
            atomicAdd(&a.rec.del_qual[gp], indelMq + 1);
            atomicAdd(&a.rec.q_sum[gp], (hasQual ? (int32_t)(int8_t)rqual[readOffset] : P.default_qual));
            atomicAdd(&a.rec.deletions[gp], 1);
            const unsigned long long slot = my_slot;
            wrote = true;
            if ((int64_t)slot < a.event_cap) {
              Event e;
              e.gpos = gp; e.read = i; e.region = C.region; e.len = len; e.roff = rloc;
              e.kind_rot = (int32_t)0x80000000;
              e.key = 0;
              e.sp = -1;
              a.events[slot] = e;
            }
          }
        }
      next_op:
        if ((op == 1 || op == 2) && !wrote && (int64_t)my_slot < a.event_cap) a.events[my_slot].gpos = -1;
        if (op == 0 || op == 1 || op == 4 || op == 7 || op == 8) readOffset += len;
        if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) refOffset += len;
      }
    }
    ChunkStats& cs = a.chunk_stats[ch];
    if (bc_n) atomicAdd(&cs.base_count, bc_n);
    if (err) atomicMax(&cs.error, err);
  }
}

void launch_read_events(const EventArgs& a, int32_t chunk_begin, int32_t chunk_count, cudaStream_t s) {
  if (chunk_count <= 0) return;
  cudaMemsetAsync(a.chunk_stats + chunk_begin, 0, sizeof(ChunkStats) * (size_t)chunk_count, s);
  k_read_events<<<chunk_count * kEvPerChunk, kEvThreads, 0, s>>>(a, chunk_begin, chunk_begin + chunk_count);
  const int64_t warps = ((int64_t)chunk_count + kIndelChunks - 1) / kIndelChunks;
  k_read_indels<<<(int)((warps * 32 + kIndelThreads - 1) / kIndelThreads), kIndelThreads, 0, s>>>(
      a, chunk_begin, chunk_begin + chunk_count);
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
// Events -> contiguous per position: the scan left each position's first slot
// in ev_end; every event takes the next slot, so afterwards ev_end is the end.
__global__ void k_event_scatter(const Event* ev, const unsigned long long* n_events, int32_t* ev_end, Event* out,
                                int64_t max_events) {
  int64_t n = min((int64_t)*n_events, max_events);
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const Event e = ev[k];
    if (e.gpos < 0) continue;  // a reserved slot that got no event
    const int32_t slot = atomicAdd(&ev_end[e.gpos], 1);
    if (slot >= 0 && slot < max_events) out[slot] = e;
  }
}

void launch_event_scatter(const Event* ev, const unsigned long long* n_events, int32_t* ev_end, Event* out,
                          cudaStream_t s, int64_t max_events) {
  if (max_events <= 0) return;
  int blocks = (int)std::min<int64_t>((max_events + 255) / 256, 152 * 8);
  k_event_scatter<<<blocks, 256, 0, s>>>(ev, n_events, ev_end, out, max_events);
}

// ---------------------------------------------------------------------------
// computePhysCov as a segmented scan over call tiles (kCallTile positions),
// fused with the exclusive scan of per-position event counts (insertions +
// deletions) that groups indel events by position.
// Phase A: tile sums.  Phase B: plain scans of the tile sums (blocks, then
// the blocks), made segmented by region for coverage (seeded with each
// region's start carry) and kept global for events.  Phase C: in-tile scan,
// insertSize /= physCov, event offsets.
__device__ inline void block_scan3(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t* s_a, uint32_t* s_b,
                                   uint32_t* s_c) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t ya = __shfl_up_sync(FULL, a, o), yb = __shfl_up_sync(FULL, b, o), yc = __shfl_up_sync(FULL, c, o);
    if (lane >= o) { a += ya; b += yb; c += yc; }
  }
  if (lane == 31) { s_a[warp] = a; s_b[warp] = b; s_c[warp] = c; }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t wa = lane < nw ? s_a[lane] : 0u, wb = lane < nw ? s_b[lane] : 0u, wc = lane < nw ? s_c[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t ya = __shfl_up_sync(FULL, wa, o), yb = __shfl_up_sync(FULL, wb, o), yc = __shfl_up_sync(FULL, wc, o);
      if (lane >= o) { wa += ya; wb += yb; wc += yc; }
    }
    s_a[lane] = wa; s_b[lane] = wb; s_c[lane] = wc;
  }
  __syncthreads();
  if (warp > 0) { a += s_a[warp - 1]; b += s_b[warp - 1]; c += s_c[warp - 1]; }
  __syncthreads();
}

// Phase a: per call tile the sums of the physical-coverage and insert-size
// difference words and of the event counts (insertions + deletions).  256
// threads per 1024-position tile, four positions each (coalesced, all loads of
// a thread in flight at once), then a block reduction.
constexpr int kScanThreads = 256;
constexpr int kScanPer = kCallTile / kScanThreads;
static_assert(kScanPer * kScanThreads == kCallTile, "four positions per scan thread");

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles_a(const RegionDev* regions, const int32_t* tile_region,
                                                                Records rec, int32_t* tile_sums, int32_t tile_begin) {
  __shared__ uint32_t s_r[3][kScanThreads / 32];
  const int32_t t = tile_begin + blockIdx.x;
  const RegionDev& g = regions[tile_region[t]];
  const int32_t p0 = (t - g.call_tile0) * kCallTile;
  uint32_t va[kScanPer], vb[kScanPer], vc[kScanPer];
#pragma unroll
  for (int k = 0; k < kScanPer; k++) {
    const int32_t p = p0 + threadIdx.x + k * kScanThreads;
    va[k] = vb[k] = vc[k] = 0;
    if (p < g.size) {
      const int64_t gp = g.pos_base + p;
      va[k] = (uint32_t)rec.phys_cov[gp];
      vb[k] = (uint32_t)rec.insert_size[gp];
      vc[k] = (uint32_t)rec.insertions[gp] + (uint32_t)rec.deletions[gp];
    }
  }
  uint32_t a = 0, b = 0, c = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; k++) { a += va[k]; b += vb[k]; c += vc[k]; }
  a = __reduce_add_sync(FULL, a);
  b = __reduce_add_sync(FULL, b);
  c = __reduce_add_sync(FULL, c);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { s_r[0][warp] = a; s_r[1][warp] = b; s_r[2][warp] = c; }
  __syncthreads();
  if (threadIdx.x < 3) {
    uint32_t v = 0;
    for (int w = 0; w < kScanThreads / 32; w++) v += s_r[threadIdx.x][w];
    tile_sums[3 * t + threadIdx.x] = (int32_t)v;
  }
}

// Phase b: plain exclusive scans of the tiles' three sums (32-bit, wrapping) over
// [t0, t0 + tn): within blocks of 1024 tiles by one CTA each, then over the
// blocks' totals by one CTA; then k_scan_tiles_b3 turns the plain prefixes
// into the region-segmented ones: the prefix at a tile minus the prefix at its
// region's first tile, plus the region's physCovStart / insertSizeStart
// (wrapping arithmetic keeps every difference exact).
__device__ inline void block_excl_scan3(uint32_t (&v)[3], uint32_t (&tot)[3], uint32_t (*s_w)[32]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t x[3] = {v[0], v[1], v[2]};
#pragma unroll
  for (int k = 0; k < 3; k++)
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(FULL, x[k], o);
      if (lane >= o) x[k] += y;
    }
  if (lane == 31)
    for (int k = 0; k < 3; k++) s_w[k][warp] = x[k];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      uint32_t w = lane < nw ? s_w[k][lane] : 0u;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, w, o);
        if (lane >= o) w += y;
      }
      if (lane < nw) s_w[k][lane] = w;  // inclusive over the warps
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const uint32_t before = warp > 0 ? s_w[k][warp - 1] : 0u;
    tot[k] = s_w[k][nw - 1];
    v[k] = before + x[k] - v[k];  // exclusive
  }
  __syncthreads();  // s_w is read by every thread before it is reused
}

__global__ void __launch_bounds__(1024) k_scan_tiles_b(int32_t* ts, int32_t* bsum, int32_t t0, int32_t tn) {
  __shared__ uint32_t s_w[3][32];
  const int32_t i = blockIdx.x * 1024 + threadIdx.x;
  uint32_t v[3], tot[3];
#pragma unroll
  for (int k = 0; k < 3; k++) v[k] = i < tn ? (uint32_t)ts[3 * (int64_t)(t0 + i) + k] : 0u;
  block_excl_scan3(v, tot, s_w);
  if (i < tn)
    for (int k = 0; k < 3; k++) ts[3 * (int64_t)(t0 + i) + k] = (int32_t)v[k];
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; k++) bsum[3 * blockIdx.x + k] = (int32_t)tot[k];
}

// the exclusive scan of the nb blocks' totals, 1024 at a time with a carry
__global__ void __launch_bounds__(1024) k_scan_tiles_b2(int32_t* bsum, int32_t nb) {
  __shared__ uint32_t s_w[3][32];
  uint32_t carry[3] = {0u, 0u, 0u};
  for (int32_t base = 0; base < nb; base += 1024) {
    const int32_t i = base + threadIdx.x;
    uint32_t v[3], tot[3];
#pragma unroll
    for (int k = 0; k < 3; k++) v[k] = i < nb ? (uint32_t)bsum[3 * i + k] : 0u;
    block_excl_scan3(v, tot, s_w);
    if (i < nb)
      for (int k = 0; k < 3; k++) bsum[3 * i + k] = (int32_t)(carry[k] + v[k]);
    for (int k = 0; k < 3; k++) carry[k] += tot[k];
  }
}

// Per tile its region-segmented exclusive prefixes into seg: the plain prefix
// (its offset in its block plus the block's) minus the plain prefix at its
// region's first tile, plus the region's start values; the event count stays
// plain (event slots are global).
__global__ void __launch_bounds__(256) k_scan_tiles_b3(const RegionDev* regions, const int32_t* tile_region,
                                                        const StatsDev* stats, const int32_t* ts, const int32_t* bsum,
                                                        int32_t* seg, int32_t t0, int32_t tn) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= tn) return;
  const int32_t t = t0 + i;
  const int32_t r = tile_region[t];
  const int32_t h = regions[r].call_tile0;  // the region's first tile (>= t0)
  auto plain = [&](int32_t tt, int k) {
    return (uint32_t)ts[3 * (int64_t)tt + k] + (uint32_t)bsum[3 * ((tt - t0) >> 10) + k];
  };
  seg[3 * (int64_t)t] = (int32_t)(plain(t, 0) - plain(h, 0) + (uint32_t)stats[r].phys_cov_start);
  seg[3 * (int64_t)t + 1] = (int32_t)(plain(t, 1) - plain(h, 1) + (uint32_t)stats[r].insert_size_start);
  seg[3 * (int64_t)t + 2] = (int32_t)plain(t, 2);
}

// Phase c: the inclusive scan inside each tile plus the tile's prefix from
// phase b, then insertSize /= physCov where physCov > 0 (S/PileUpRegion.scala:
// 90-100), and each position's first event slot.  The tile's words are loaded
// coalesced into shared memory, each thread scans four consecutive positions,
// a block scan joins the threads, and the results go back coalesced.
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles_c(const RegionDev* regions, const int32_t* tile_region,
                                                                Records rec, const int32_t* tile_sums,
                                                                int32_t tile_begin) {
  __shared__ __align__(16) uint32_t s_v[3][kCallTile];
  __shared__ uint32_t s_a[32], s_b[32], s_c[32];
  const int32_t t = tile_begin + blockIdx.x;
  const RegionDev& g = regions[tile_region[t]];
  const int32_t p0 = (t - g.call_tile0) * kCallTile;
  const int32_t n = min(kCallTile, g.size - p0);
#pragma unroll
  for (int k = 0; k < kScanPer; k++) {
    const int32_t i = threadIdx.x + k * kScanThreads;
    uint32_t a = 0, b = 0, c = 0;
    if (i < n) {
      const int64_t gp = g.pos_base + p0 + i;
      a = (uint32_t)rec.phys_cov[gp];
      b = (uint32_t)rec.insert_size[gp];
      c = (uint32_t)rec.insertions[gp] + (uint32_t)rec.deletions[gp];
    }
    s_v[0][i] = a; s_v[1][i] = b; s_v[2][i] = c;
  }
  __syncthreads();
  // positions 4 * tid .. 4 * tid + 3
  const uint4 xa = reinterpret_cast<const uint4*>(s_v[0])[threadIdx.x];
  const uint4 xb = reinterpret_cast<const uint4*>(s_v[1])[threadIdx.x];
  const uint4 xc = reinterpret_cast<const uint4*>(s_v[2])[threadIdx.x];
  uint32_t a = xa.x + xa.y + xa.z + xa.w, b = xb.x + xb.y + xb.z + xb.w, c = xc.x + xc.y + xc.z + xc.w;
  const uint32_t ta = a, tb = b, tc = c;
  block_scan3(a, b, c, s_a, s_b, s_c);  // inclusive over threads
  // exclusive prefix of this thread's first position, with the tile's prefix
  uint32_t pa = a - ta + (uint32_t)tile_sums[3 * t], pb = b - tb + (uint32_t)tile_sums[3 * t + 1];
  uint32_t pc = c - tc + (uint32_t)tile_sums[3 * t + 2];
  const uint32_t ea[4] = {xa.x, xa.y, xa.z, xa.w}, eb[4] = {xb.x, xb.y, xb.z, xb.w}, ec[4] = {xc.x, xc.y, xc.z, xc.w};
  uint32_t oa[4], ob[4], oc[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    oc[j] = ec[j] ? pc : 0xffffffffu;  // first event slot of the position, or none
    pa += ea[j]; pb += eb[j]; pc += ec[j];
    int32_t cov = (int32_t)pa, is = (int32_t)pb;
    if (cov > 0) is = is / cov;
    oa[j] = (uint32_t)cov; ob[j] = (uint32_t)is;
  }
  __syncthreads();  // every thread has read its words
  reinterpret_cast<uint4*>(s_v[0])[threadIdx.x] = make_uint4(oa[0], oa[1], oa[2], oa[3]);
  reinterpret_cast<uint4*>(s_v[1])[threadIdx.x] = make_uint4(ob[0], ob[1], ob[2], ob[3]);
  reinterpret_cast<uint4*>(s_v[2])[threadIdx.x] = make_uint4(oc[0], oc[1], oc[2], oc[3]);
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanPer; k++) {
    const int32_t i = threadIdx.x + k * kScanThreads;
    if (i < n) {
      const int64_t gp = g.pos_base + p0 + i;
      rec.phys_cov[gp] = (int32_t)s_v[0][i];
      rec.insert_size[gp] = (int32_t)s_v[1][i];
      if (s_v[2][i] != 0xffffffffu) rec.ev_end[gp] = (int32_t)s_v[2][i];  // first slot
    }
  }
}

void launch_physcov_scan(const RegionDev* regions, const int32_t* call_tile_region, int32_t tile_begin,
                         int32_t n_tiles, Records rec, const StatsDev* stats, int32_t* tile_sums, int32_t* seg,
                         int32_t* block_sums, int32_t region_begin, int32_t n_regions, cudaStream_t s) {
  (void)region_begin;
  (void)n_regions;
  if (n_tiles <= 0) return;
  const int32_t nb = (n_tiles + 1023) / 1024;
  k_scan_tiles_a<<<n_tiles, kScanThreads, 0, s>>>(regions, call_tile_region, rec, tile_sums, tile_begin);
  k_scan_tiles_b<<<nb, 1024, 0, s>>>(tile_sums, block_sums, tile_begin, n_tiles);
  k_scan_tiles_b2<<<1, 1024, 0, s>>>(block_sums, nb);
  k_scan_tiles_b3<<<(n_tiles + 255) / 256, 256, 0, s>>>(regions, call_tile_region, stats, tile_sums, block_sums, seg,
                                                        tile_begin, n_tiles);
  k_scan_tiles_c<<<n_tiles, kScanThreads, 0, s>>>(regions, call_tile_region, rec, seg, tile_begin);
}

// ---------------------------------------------------------------------------
// minDepth of GenomeRegion.postProcess (S/GenomeRegion.scala:216-224).
__device__ inline int64_t java_round(double x) {
  double f = floor(x);
  return (int64_t)((x - f >= 0.5) ? f + 1.0 : f);
}

__device__ inline int32_t region_min_depth(const DevParams& P, unsigned long long base_count, int32_t size) {
  // minDepth of GenomeRegion.postProcess (S/GenomeRegion.scala:216-224)
  const int64_t meanCoverage = roundDivL((int64_t)base_count, size);
  if (P.min_depth >= 1) return (int32_t)P.min_depth;
  return max((int32_t)java_round(P.min_depth * (double)meanCoverage), P.min_min_depth);
}

// `per` CTAs per region, each adding up a share of the region's per-chunk
// partial statistics; with one CTA it stores them, with several each adds its
// sums with atomics and the CTA that finishes last (a counter in the region's
// statistics, after a fence) computes minDepth.
constexpr int kPrepThreads = 256, kPrepChunksPerCta = 512;
__global__ void __launch_bounds__(kPrepThreads) k_region_prep(const RegionDev* regions, StatsDev* stats,
                                                               const ChunkStats* cs, DevParams P, int32_t per) {
  __shared__ unsigned long long s_u[8];
  __shared__ int32_t s_i[3];
  const int32_t r = blockIdx.x / per, part = blockIdx.x % per;
  const RegionDev& g = regions[r];
  const int32_t span = (g.n_chunks + per - 1) / per;
  const int32_t k0 = g.chunk0 + part * span, k1 = min(g.chunk0 + g.n_chunks, k0 + span);
  unsigned long long u[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  uint32_t pcs = 0, iss = 0;
  int32_t err = 0;
  for (int32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    const ChunkStats c = cs[k];
    u[0] += c.read_count; u[1] += c.base_count; u[2] += c.fr_count; u[3] += c.fr_sum;
    u[4] += c.fr_sumsq; u[5] += c.rf_count; u[6] += c.rf_sum; u[7] += c.rf_sumsq;
    pcs += (uint32_t)c.phys_cov_start;
    iss += (uint32_t)c.insert_size_start;
    err = max(err, c.error);
  }
  if (threadIdx.x < 8) s_u[threadIdx.x] = 0;
  if (threadIdx.x < 3) s_i[threadIdx.x] = 0;
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const unsigned long long v = warp_sum_u64(u[k]);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&s_u[k], v);
  }
  pcs = __reduce_add_sync(FULL, pcs);
  iss = __reduce_add_sync(FULL, iss);
  err = __reduce_max_sync(FULL, err);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_i[0], (int32_t)pcs);
    atomicAdd(&s_i[1], (int32_t)iss);
    atomicMax(&s_i[2], err);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    StatsDev& st = stats[r];
    if (per == 1) {
      st.read_count = s_u[0];
      st.base_count += s_u[1];  // the walk kernel added the aligned bases already
      st.fr_count = s_u[2]; st.fr_sum = s_u[3]; st.fr_sumsq = s_u[4];
      st.rf_count = s_u[5]; st.rf_sum = s_u[6]; st.rf_sumsq = s_u[7];
      st.phys_cov_start = s_i[0];
      st.insert_size_start = s_i[1];
      st.error = s_i[2];
      st.min_depth = region_min_depth(P, st.base_count, g.size);
    } else {  // the statistics start at zero (base_count at the walk's aligned bases)
      atomicAdd(&st.read_count, s_u[0]);
      atomicAdd(&st.base_count, s_u[1]);
      atomicAdd(&st.fr_count, s_u[2]); atomicAdd(&st.fr_sum, s_u[3]); atomicAdd(&st.fr_sumsq, s_u[4]);
      atomicAdd(&st.rf_count, s_u[5]); atomicAdd(&st.rf_sum, s_u[6]); atomicAdd(&st.rf_sumsq, s_u[7]);
      atomicAdd(&st.phys_cov_start, s_i[0]);
      atomicAdd(&st.insert_size_start, s_i[1]);
      atomicMax(&st.error, s_i[2]);
      __threadfence();
      if (atomicAdd(&st.prep_done, 1) == per - 1) {  // every other part has added its sums
        __threadfence();
        st.min_depth = region_min_depth(P, atomicAdd(&st.base_count, 0ull), g.size);
      }
    }
  }
}

void launch_region_prep(const RegionDev* regions, StatsDev* stats, const ChunkStats* chunk_stats,
                        int32_t n_regions, int32_t max_chunks, DevParams P, cudaStream_t s) {
  if (n_regions == 0) return;
  const int32_t per = std::max(1, (max_chunks + kPrepChunksPerCta - 1) / kPrepChunksPerCta);
  k_region_prep<<<n_regions * per, kPrepThreads, 0, s>>>(regions, stats, chunk_stats, P, per);
}

}  // namespace pg
