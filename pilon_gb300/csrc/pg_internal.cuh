// pg_internal.cuh — device data layout, shared device functions and kernel
// entry points of the pilon_gb300 engine.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pilon_gb300.h"

namespace pg {

// ---------------------------------------------------------------------------
// Layout in HBM
//
// Positions of all regions of one pg_pileup_regions call are concatenated
// ("global positions"); region r owns [pos_base[r], pos_base[r] + size_r).
// The pileup record of a position is structure-of-arrays:
//   count     int4      A,C,G,T base counts           (PileUp.baseCount)
//   qual_sum  int64[4]  A,C,G,T qual*(mq+1) sums      (PileUp.qualSum)
//   mq_sum, q_sum, bad_pair, clips, deletions, del_qual, insertions,
//   ins_qual  int32                                   (PileUp Int fields)
//   phys_cov, insert_size int32: difference arrays during the walk, final
//             values after the scan                   (PileUp.physCov/insertSize)
// = 88 bytes per position, written once by the walk kernel.
// Calls: call (uint32 PG_CALL_* flags), score (int64), indel_len (int32),
// ins_str (int32 offset into the insertion-string pool or -1).
// ---------------------------------------------------------------------------

struct Reads {  // device pointers of the read store
  int64_t n;
  const int32_t *pos, *aend, *tlen, *ref_id, *mate_ref_id, *l_seq;
  const uint16_t *flag, *n_cigar;
  const uint8_t *mapq, *seq, *qual;
  const int64_t *cigar_off, *seq_off, *qual_off;
  const uint32_t *cigar;
  int64_t n_cigar_words, seq_bytes, qual_bytes;
  // Per-read walk descriptor, two int4 per read, made once per read store by
  // k_read_extent (everything of PileUpRegion.addRead's setup that does not
  // depend on the region or the options):
  //   d0 = {pos, end (alignment end, or pos when unmapped), ref_id, adjMq + 1}
  //   d1 = {lead | trail << 16, mlen | hasQual << 30 | simple << 31,
  //         (pos - first touched position) | pairOk << 30, last touched position - pos}
  // simple: the CIGAR is [H][S] M|=|X [S][H] with clips < 65536 and 0 <= adjMq <= 255;
  // a read that is not simple has d1.x = 1 when its CIGAR holds an I or D, else 0.
  const int4* desc;
  // Walk entries, made once per read store by k_entry_fill: one per M/=/X or S
  // operator of every read, in read order; the entries of read i are
  // [entry_off[i], entry_off[i + 1]).  Three int4 per entry:
  //   e0 = {pos, end (alignment end, or pos when unmapped), first locus of the
  //         operator (S: clipStart of S/PileUpRegion.scala:195), length}
  //   e1 = {read offset of the operator, read length, adjMq + 1, meta}
  //   e2 = {qual_off + read offset (int64), 2 * seq_off + read offset (int64, a nibble index)}
  //   meta = mapq | (flag >> 8 & 7) << 8 (secondary, qc-fail, duplicate) |
  //          kEntClip | kEntHasQual | kEntPairOk
  const int4* entries;
  const int64_t* entry_off;   // n + 1 offsets
};
constexpr uint32_t kDescHasQual = 1u << 30, kDescSimple = 1u << 31, kDescPairOk = 1u << 30;
constexpr uint32_t kEntClip = 1u << 11, kEntHasQual = 1u << 12, kEntPairOk = 1u << 13;

struct RegionDev {       // per region, device copy
  int32_t contig, start, stop, size;
  int32_t chunk0, n_chunks;  // read chunks of this region
  int64_t pos_base;      // first global position
  int64_t ref_off;       // offset of the contig in the concatenated reference
  int64_t contig_len;
  int64_t read_begin, read_end;
  int32_t qs, qe;        // query window of BamFile.process
  int32_t walk_tile0, n_walk_tiles;
  int32_t call_tile0, n_call_tiles;
};

struct StatsDev {        // per region, accumulated on the device
  unsigned long long base_count;
  unsigned long long read_count;
  int32_t phys_cov_start, insert_size_start;
  int32_t min_depth, n_changes;
  unsigned long long fr_count, fr_sum, fr_sumsq, rf_count, rf_sum, rf_sumsq;
  int32_t error;
  int32_t n_ins;
  int32_t prep_done;     // CTAs of k_region_prep that have added their part
  int32_t range_error;   // 1: the region's read range holds reads of another reference
};

struct WalkTile {
  int32_t region, lo, len, pad;
  int64_t ent_lo, ent_hi;  // walk entries of the reads that can touch the tile
};

struct ReadChunk {       // reads [lo, hi) fed to region `region`
  int32_t region, pad;
  int64_t lo, hi;
};

struct ChunkStats {      // per read chunk: partial sums of the region statistics
  unsigned long long read_count, base_count, fr_count, fr_sum, fr_sumsq, rf_count, rf_sum, rf_sumsq;
  int32_t phys_cov_start, insert_size_start, error;
  int32_t n_indel;       // reads of the chunk with I/D operators, listed for k_read_indels
};

struct Event {           // one insertion or deletion added to a pileup
  int64_t gpos;
  int64_t read;
  uint64_t key;          // insertions: 4-bit codes of the (rotated) string, characters 0..15
  int64_t sp;            // insertions longer than 16: characters 16.. packed 16 per word in the string pool
  int32_t region;
  int32_t len;
  int32_t roff;          // read offset of the indel (insertions)
  int32_t kind_rot;      // bit 31: deletion; low bits: right rotation of the insertion
};

struct Cand {            // change candidate of pass 1, in position order
  int64_t gpos;
  int32_t region, p, kind, len;
};

struct Records {
  int4 *count;
  longlong2 *qual_sum;   // two longlong2 per position
  int32_t *mq_sum, *q_sum, *bad_pair, *clips, *deletions, *del_qual, *insertions, *ins_qual;
  int32_t *phys_cov, *insert_size;
  int32_t *ev_end;       // events of a position: [ev_end - (insertions + deletions), ev_end)
  uint32_t *call;
  int64_t *score;
  int32_t *indel_len, *ins_str;
};

struct ReadExtent {      // maxima over the read store, for tile read ranges
  int32_t max_lead;      // max(pos - first touched position)
  int32_t max_back;      // max(last touched position - pos)
  unsigned long long n_indel_ops;
  unsigned long long bad_read;  // 1 + index of a read whose offsets leave their arrays, else 0
  int32_t unsorted;      // 1 if positions decrease within one reference
  // 1 if the references are not in one run each: a reference id below the one
  // before it, or a placed read after an unplaced one (negative id).  A
  // coordinate-sorted BAM has each reference in one run, unplaced reads last.
  int32_t ungrouped;
  int32_t max_span;      // max(aend - pos + 1): how far before a window a read that overlaps it can start
  // reads with simple CIGARs and qualities, by adjusted mq + 1 (1..256); the
  // walk adds the reads of the most common value with one atomic per base
  unsigned int mq1_hist[257];
};

struct DevParams {
  int32_t min_mq, min_qual, flank, default_qual, min_min_depth;
  int32_t nonpf, duplicates, old_indel, fix_amb, long_read, bam_type, long_read_only;
  double min_depth;
  int32_t huge;          // 5 * maxInsertSizes(bamType) (S/BamFile.scala:192)
};

constexpr int kCallTile = 1024;     // positions per call / scan tile
constexpr int kReadsPerChunk = 256;   // one read per thread of k_read_events
// Reads one walk pass adds to a tile.  At most 4095 reads per position keep the
// packed shared counters exact: sum of qual (20 bits) + count (12 bits) in one
// word for qualities up to 256 (the API keeps defaultQual within a byte; a
// larger one would lower the pass size here, never to 0), and the
// qual * (mq + 1 - M) sums within int32.
constexpr int64_t kMaxReadsPerPass = 4095;
inline int32_t walk_reads_per_pass(int32_t default_qual) {
  const int32_t q = default_qual > 127 ? default_qual : 127;
  const int64_t n = kMaxReadsPerPass < 1048575 / q ? kMaxReadsPerPass : 1048575 / q;
  return (int32_t)(n > 0 ? n : 1);  // a pass always advances
}

// ---- Java integer helpers (wrapping Int, truncating division) -------------
__host__ __device__ inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__host__ __device__ inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
__host__ __device__ inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
__host__ __device__ inline int32_t roundDivI(int32_t n, int32_t d) { return d > 0 ? wadd(n, d / 2) / d : 0; }
__host__ __device__ inline int64_t roundDivL(int64_t n, int64_t d) { return d > 0 ? (n + d / 2) / d : 0; }
__host__ __device__ inline int32_t pctI(int32_t n, int32_t d) { return roundDivI(wmul(100, n), d); }

__device__ inline int nib_index(uint32_t nib) {  // BAM code -> A,C,G,T index or -1
  return nib == 1 ? 0 : nib == 2 ? 1 : nib == 4 ? 2 : nib == 8 ? 3 : -1;
}
__device__ inline uint8_t nib_char(uint32_t nib) {
  const char* t = "=ACMGRSVTWYHKDBN";
  return (uint8_t)t[nib & 15];
}
__device__ inline uint8_t upper(uint8_t c) { return (c >= 'a' && c <= 'z') ? (uint8_t)(c - 32) : c; }

// Non-negative a / positive b, in 32 bits when both fit (same result).
__device__ inline int64_t div_s64(int64_t a, int64_t b) {
  if ((uint64_t)a <= 0xffffffffull && (uint64_t)b <= 0xffffffffull) return (int64_t)((uint32_t)a / (uint32_t)b);
  return a / b;
}

// ---- Per-position call (PileUp.BaseCall, S/PileUp.scala:132-255) -----------
struct PosRec {
  int64_t cnt[4], qs[4];
  int32_t mq_sum, q_sum, deletions, del_qual, insertions, ins_qual;
};

__device__ inline void load_rec(const Records& Rc, int64_t gp, PosRec& r) {
  int4 c = Rc.count[gp];
  r.cnt[0] = c.x; r.cnt[1] = c.y; r.cnt[2] = c.z; r.cnt[3] = c.w;
  longlong2 a = Rc.qual_sum[2 * gp], b = Rc.qual_sum[2 * gp + 1];
  r.qs[0] = a.x; r.qs[1] = a.y; r.qs[2] = b.x; r.qs[3] = b.y;
  r.mq_sum = Rc.mq_sum[gp]; r.q_sum = Rc.q_sum[gp];
  r.deletions = Rc.deletions[gp]; r.del_qual = Rc.del_qual[gp];
  r.insertions = Rc.insertions[gp]; r.ins_qual = Rc.ins_qual[gp];
}

// v[i] for a run-time i without dynamic indexing (keeps the array in registers)
__device__ inline int64_t pick4(const int64_t v[4], int i) {
  return i == 0 ? v[0] : i == 1 ? v[1] : i == 2 ? v[2] : v[3];
}

// Stable descending order of four sums: first and second index.
__device__ inline void order2(const int64_t v[4], int& o0, int& o1) {
  o0 = 0;
  int64_t m0 = v[0];
#pragma unroll
  for (int i = 1; i < 4; i++)
    if (v[i] > m0) { o0 = i; m0 = v[i]; }
  o1 = -1;
  int64_t m1 = 0;
#pragma unroll
  for (int i = 0; i < 4; i++)
    if (i != o0 && (o1 < 0 || v[i] > m1)) { o1 = i; m1 = v[i]; }
}

__device__ inline int32_t pick4_32(const int32_t v[4], int i) {
  return i == 0 ? v[0] : i == 1 ? v[1] : i == 2 ? v[2] : v[3];
}
__device__ inline void order2_32(const int32_t v[4], int& o0, int& o1) {  // order2 on 32-bit sums
  o0 = 0;
  int32_t m0 = v[0];
#pragma unroll
  for (int i = 1; i < 4; i++)
    if (v[i] > m0) { o0 = i; m0 = v[i]; }
  o1 = -1;
  int32_t m1 = 0;
#pragma unroll
  for (int i = 0; i < 4; i++)
    if (i != o0 && (o1 < 0 || v[i] > m1)) { o1 = i; m1 = v[i]; }
}

struct CallCtx {         // what the indel vote needs
  const Event* ev;       // events grouped by position
  int64_t ev_lo, ev_hi;  // this position's events (clamped to the buffer)
  const uint64_t* spool; // packed tails of insertions longer than 16
  const uint8_t* ref;    // concatenated reference
  int64_t ref_off;       // contig offset
  int64_t contig_len;
  char* pool;            // insertion-string pool
  unsigned long long* pool_fill;
  int64_t pool_cap;
};

// character j (4-bit code) of an insertion event's string
__device__ inline uint32_t ins_char(const CallCtx& c, const Event& e, int32_t j) {
  if (j < 16) return (uint32_t)(e.key >> (60 - 4 * j)) & 15u;
  const int32_t t = j - 16;
  return (uint32_t)(c.spool[e.sp + (t >> 4)] >> (60 - 4 * (t & 15))) & 15u;
}

__device__ inline bool same_indel(const CallCtx& c, const Event& a, const Event& b) {
  if (a.len != b.len) return false;
  if (a.kind_rot < 0) return true;  // deletions at one position: same length = same reference slice
  if (a.key != b.key) return false;
  for (int32_t w = 0; w < (a.len - 16 + 15) / 16; w++)  // tail words (none when len <= 16)
    if (c.spool[a.sp + w] != c.spool[b.sp + w]) return false;
  return true;
}

// Majority vote of hetIndelCall (S/PileUp.scala:209-247): returns the event
// index of the winner, or -1.  The winner needs count >= 2 and a strict
// majority, so the result does not depend on event order.
__device__ inline int64_t indel_vote(const CallCtx& c, int64_t gp, bool del) {
  int64_t cand = -1;
  int64_t cnt = 0, total = 0;
  for (int64_t k = c.ev_lo; k < c.ev_hi; k++) {
    const Event& e = c.ev[k];
    if ((e.kind_rot < 0) != del) continue;
    total++;
    if (cnt == 0) { cand = k; cnt = 1; }
    else if (same_indel(c, e, c.ev[cand])) cnt++;
    else cnt--;
  }
  if (cand < 0) return -1;
  int64_t win = 0;
  for (int64_t k = c.ev_lo; k < c.ev_hi; k++) {
    const Event& e = c.ev[k];
    if ((e.kind_rot < 0) != del) continue;
    if (same_indel(c, e, c.ev[cand])) win++;
  }
  if (win < 2 || win <= total / 2) return -1;
  return cand;
}

__device__ inline bool insertion_has_n(const CallCtx& c, const Event& e) {
  for (int32_t j = 0; j < e.len; j++)
    if (ins_char(c, e, j) == 15u) return true;  // 'N'
  return false;
}

struct CallOut {
  uint32_t flags;  // base/alt/homo/indel bits only
  int64_t score;
  int32_t indel_len;
  int64_t win_event;  // winner event (insertion) or -1
};

// dloc0 = 0-based contig index of position p's locus minus one (locus - 1).
__device__ inline CallOut base_call(const PosRec& r, const DevParams& P, const CallCtx& c, int64_t gp,
                                    int64_t locus0) {
  CallOut o;
  int64_t n = r.cnt[0] + r.cnt[1] + r.cnt[2] + r.cnt[3];
  int o0, o1;
  bool homo;
  int64_t diff;
  if ((uint64_t)(r.qs[0] | r.qs[1] | r.qs[2] | r.qs[3]) < (1ull << 29)) {
    // every quality sum in [0, 2^29): the same arithmetic in 32 bits (the
    // total stays below 2^31, the scores within [-total, total])
    const int32_t q[4] = {(int32_t)r.qs[0], (int32_t)r.qs[1], (int32_t)r.qs[2], (int32_t)r.qs[3]};
    const int32_t c[4] = {(int32_t)r.cnt[0], (int32_t)r.cnt[1], (int32_t)r.cnt[2], (int32_t)r.cnt[3]};
    if (r.q_sum > 0) order2_32(q, o0, o1); else order2_32(c, o0, o1);
    const int32_t baseSum = pick4_32(q, o0), altBaseSum = pick4_32(q, o1);
    const int32_t total = q[0] + q[1] + q[2] + q[3];
    const int32_t homoScore = baseSum - (total - baseSum);
    const int32_t half = total / 2;
    const int32_t d1 = half - baseSum, d2 = half - altBaseSum;
    const int32_t heteroScore = total - abs(d1) - abs(d2);
    homo = homoScore >= heteroScore;
    diff = (int64_t)homoScore - (int64_t)heteroScore;
  } else {
    if (r.q_sum > 0) order2(r.qs, o0, o1); else order2(r.cnt, o0, o1);
    int64_t baseSum = pick4(r.qs, o0), altBaseSum = pick4(r.qs, o1);
    int64_t total = r.qs[0] + r.qs[1] + r.qs[2] + r.qs[3];
    int64_t homoScore = baseSum - (total - baseSum);
    int64_t half = total / 2;
    int64_t d1 = half - baseSum, d2 = half - altBaseSum;
    int64_t heteroScore = total - (d1 < 0 ? -d1 : d1) - (d2 < 0 ? -d2 : d2);
    homo = homoScore >= heteroScore;
    diff = homoScore - heteroScore;
  }
  if (diff < 0) diff = -diff;
  o.score = r.mq_sum > 0 ? div_s64(diff * n, (int64_t)r.mq_sum) : 0;
  o.flags = (uint32_t)o0 | ((uint32_t)o1 << 2);
  if (n > 0) o.flags |= PG_CALL_HAS_BASE;
  if (homo) o.flags |= PG_CALL_HOMO;
  o.indel_len = 0;
  o.win_event = -1;
  int64_t depth = n + r.deletions;
  int32_t cnt32 = (int32_t)n;
  bool indelCalled = false, homoIndel = true;
  for (int pass = 0; pass < 2 && !indelCalled; pass++) {
    bool del = pass == 1;
    bool gate = del ? (r.deletions > 2 && r.deletions > r.insertions)
                    : (r.insertions > 2 && r.insertions > r.deletions);
    if (!gate) continue;
    int32_t pct = del ? max(pctI(r.del_qual, r.mq_sum), pctI(r.deletions, wadd(cnt32, r.deletions)))
                      : max(pctI(r.ins_qual, r.mq_sum), pctI(r.insertions, cnt32));
    if (depth < P.min_min_depth || pct < 5) continue;
    int64_t w = indel_vote(c, gp, del);
    if (w < 0) continue;
    const Event& e = c.ev[w];
    int32_t len = e.len;
    bool hasN = false;
    if (del) {
      // deletion string = reference bytes [dloc-1, dloc-1+len) of the contig
      for (int32_t j = 0; j < len; j++) {
        int64_t k = locus0 + j;
        if (k >= 0 && k < c.contig_len && c.ref[c.ref_off + k] == 'N') hasN = true;
      }
    } else {
      hasN = insertion_has_n(c, e);
    }
    if (hasN) continue;
    bool call = false, homoI = true;
    if (P.old_indel) {
      if (pct >= 33 && pct >= 50 - len) { call = true; homoI = true; }
    } else {
      int32_t middle = max(45 - len, 10);
      int32_t low = middle / 2;
      int32_t high = middle + middle - low;
      if (pct > high) { call = true; homoI = true; }
      else if (pct >= low) { call = true; homoI = false; }
    }
    if (call) {
      indelCalled = true;
      homoIndel = homoI;
      o.indel_len = len;
      o.flags |= del ? PG_CALL_DEL : PG_CALL_INS;
      if (!del) o.win_event = w;
    }
  }
  if (homoIndel) o.flags |= PG_CALL_HOMO_INDEL;
  return o;
}

// Writes the winning insertion's characters into the pool; returns the offset.
__device__ inline int32_t pool_insertion(const CallCtx& c, const Event& e) {
  unsigned long long off = atomicAdd(c.pool_fill, (unsigned long long)e.len);
  if ((int64_t)(off + e.len) > c.pool_cap) return -2;  // overflow: host grows and reruns
  for (int32_t j = 0; j < e.len; j++) c.pool[off + j] = (char)nib_char(ins_char(c, e, j));
  return (int32_t)off;
}

// ---- kernels ----------------------------------------------------------------
struct WalkArgs {
  Reads R;
  const RegionDev* regions;
  const WalkTile* tiles;
  int32_t n_tiles;
  Records rec;
  StatsDev* stats;
  DevParams P;
  const uint8_t* ref;
  int32_t tile_width;
  int32_t packed;        // walk variant: lanes per simple read, 0 = 32, 1 = 16, 2 = 8
  uint32_t mode_mq1;     // the read store's most common adjusted mq + 1 (any value gives the same sums)
  int32_t reads_per_pass;  // reads one walk pass adds to a tile (kMaxReadsPerPass or fewer)
};

struct EventArgs {
  Reads R;
  const RegionDev* regions;
  const ReadChunk* chunks;
  int32_t n_chunks;
  Records rec;
  StatsDev* stats;
  DevParams P;
  const uint8_t* ref;
  Event* events;
  unsigned long long* n_events;
  int64_t event_cap;
  ChunkStats* chunk_stats;
  uint64_t* spool;                 // insertion tails, 16 characters per word
  unsigned long long* spool_fill;
  int64_t spool_cap;
  int64_t* indel_list;             // per chunk kReadsPerChunk slots: its reads with I/D
};

// Per call tile, written by k_call_desc once the region statistics exist:
// what k_call needs of the tile's region, so that a unit of the call needs one
// descriptor load instead of the tile -> region -> statistics chain.
struct __align__(16) CallDesc {
  int64_t gp0;         // global position of the tile's first position
  int64_t ref_off;     // the contig's offset in the concatenated reference
  int64_t contig_len;
  int32_t start;       // the region's first locus
  int32_t p0;          // region index of the tile's first position
  int32_t n;           // positions of the tile
  int32_t min_depth;   // the region's minDepth
  int32_t reads;       // 1 when reads were fed to the region
  int32_t pad;
};
static_assert(sizeof(CallDesc) == 48, "call tile descriptor");

struct CallArgs {
  Reads R;
  const RegionDev* regions;
  const int32_t* call_tile_region;  // region of each call tile
  CallDesc* call_desc;              // per call tile (k_call_desc)
  int32_t n_call_tiles;
  Records rec;
  StatsDev* stats;
  DevParams P;
  const uint8_t* ref;
  const Event* ev_sorted;     // grouped by position (Records::ev_end)
  int64_t event_cap;
  const uint64_t* spool;
  int32_t* cand_count;        // per call tile
  char* pool;
  unsigned long long* pool_fill;
  int64_t pool_cap;
};

void launch_read_extent(const Reads& R, ReadExtent* out, int4* desc, cudaStream_t s);
// a packed store's per-read lengths (for the offset scans) and alignment ends
void launch_packed_lengths(const Reads& R, int64_t* cig, int64_t* seq, int64_t* qual, cudaStream_t s);
void launch_packed_aend(const Reads& R, int32_t* aend, cudaStream_t s);
// Builds R.entry_off (n + 1 int64; `sums` holds (n + 1) / 1024 + 2 int64 of
// scan scratch) and R.entries (3 int4 per entry), after the store passed
// k_read_extent's checks.  Returns nothing: the host reads entry_off[n].
void launch_entry_count(const Reads& R, int64_t* entry_off, int64_t* sums, cudaStream_t s);
void launch_entry_fill(const Reads& R, const int64_t* entry_off, int4* entries, cudaStream_t s);
void launch_tile_ranges(const Reads& R, const RegionDev* regions, WalkTile* tiles, int32_t n_tiles,
                        const ReadExtent* ext, StatsDev* stats, cudaStream_t s);
void launch_walk(const WalkArgs& a, int32_t tile_begin, int32_t tile_count, int warps, cudaStream_t s);
void launch_read_events(const EventArgs& a, int32_t chunk_begin, int32_t chunk_count, cudaStream_t s);
void launch_scan_small(const int32_t* in, int32_t* out_excl, int32_t n, cudaStream_t s);
void launch_event_scatter(const Event* ev, const unsigned long long* n_events, int32_t* ev_end, Event* out,
                          cudaStream_t s, int64_t max_events);
void launch_physcov_scan(const RegionDev* regions, const int32_t* call_tile_region, int32_t tile_begin,
                         int32_t n_tiles, Records rec, const StatsDev* stats, int32_t* tile_sums, int32_t* seg,
                         int32_t* block_sums, int32_t region_begin, int32_t n_regions, cudaStream_t s);
void launch_region_prep(const RegionDev* regions, StatsDev* stats, const ChunkStats* chunk_stats,
                        int32_t n_regions, int32_t max_chunks, DevParams P, cudaStream_t s);
void launch_call(const CallArgs& a, int32_t tile_begin, int32_t n_tiles, cudaStream_t s);
void launch_cand_list(const CallArgs& a, const int32_t* cand_off, Cand* cands, int32_t cand_cap,
                      int32_t tile_begin, int32_t n_tiles, cudaStream_t s);
void launch_resolve(const RegionDev* regions, int32_t n_regions, const int32_t* cand_off, Cand* cands,
                    int32_t cand_cap, StatsDev* stats, cudaStream_t s);
void launch_apply_spans(const CallArgs& a, const Cand* cands, const int32_t* cand_total, int32_t cand_cap,
                        cudaStream_t s);
void launch_change_count(const RegionDev* regions, const int32_t* tile_region, const uint32_t* call, int32_t* count,
                         int32_t n_tiles, cudaStream_t s);
void launch_change_write(const RegionDev* regions, const int32_t* tile_region, const Records& rec,
                         const int32_t* count, const int32_t* off, pg_change* out, int32_t n_tiles, cudaStream_t s);

}  // namespace pg
