// pg_kmer.cuh — arguments of the K-mer tally kernels (pg_kmer.cu).
#pragma once
#include "pg_internal.cuh"

namespace pg {

// reads [lo, hi) of window w (or entries [lo, hi) of the read list), walked
// by one CTA of k_kmer_count
struct KmerChunk {
  int64_t lo, hi;
  int32_t w, pad;
};

// One slot of a window's table (64-bit keys, K <= 31): everything one K-mer
// event touches in one 64-byte line, the key and the counters a probe hit adds
// to in its first 32 bytes.  key = the 2-bit K-mer | 1 << 63 (0 = empty, so a
// table is cleared with zeros).  The PileUp fields buildGraph reads
// (S/Assembler.scala:132-154): baseCount (cnt), qualSum (qs, Long), qSum (an
// Int, wrapping); mqSum only weighs the score, which the graph does not use.
struct __align__(64) KmerSlot {
  unsigned long long key;
  uint32_t q_sum, pad;
  uint32_t cnt[4];
  unsigned long long qs[4];
};
// The wide slot (K <= 63): a 128-bit key (hi | 1 << 63; both words 0 = empty),
// inserted with the 16-byte compare-and-swap.
struct __align__(32) KmerSlotWide {
  unsigned long long lo, hi;
  uint32_t cnt[4];
  unsigned long long qs[4];
  uint32_t q_sum, pad[7];
};
static_assert(sizeof(KmerSlot) == 64 && sizeof(KmerSlotWide) == 96, "K-mer slot layout");

struct KmerArgs {
  Reads R;
  const int64_t* rlist;       // not null: window and chunk ranges index this list of reads
  const int32_t* win_list;    // the batch's windows (indices into the per-window arrays)
  int32_t n_win;
  int32_t K;
  int32_t min_qual, default_qual, min_depth;
  int32_t wide;               // 1: KmerSlotWide tables, 4-word exotic keys, pg_kmer_edge_wide output
  const KmerChunk* chunks;    // the batch's read chunks
  int32_t n_chunks;
  int32_t* full;              // per window: 1 when a probe sequence ran past the bound (count again, larger)
  unsigned long long* used;   // per window: distinct K-mers inserted
  // tables: slots [slot_base[w], slot_base[w] + slot_cap[w]) of window w, relative to the batch
  // (the exotic tables and event lists are relative to the pass)
  const int64_t* slot_base;
  const int64_t* slot_cap;
  void* slots;                // KmerSlot or KmerSlotWide
  // exotic tables (4-bit keys) of every window of the pass, one warp per window
  const int64_t* x_base;
  const int64_t* x_cap;
  unsigned long long* x_keys; // 2 per slot (wide: 4)
  uint8_t* x_used;
  uint32_t* x_cnt;
  unsigned long long* x_qs;
  uint32_t* x_q;
  // exotic K-mer events (read, strand << 32 | offset), listed per window by k_kmer_count
  const int64_t* x_ev_base;
  const int64_t* x_ev_cap;
  unsigned long long* x_ev_fill;
  longlong2* x_events;
  // output
  pg_kmer_edge* edges;
  pg_kmer_edge_wide* wedges;  // output of the wide tally
  int64_t edge_cap;
  unsigned long long* n_edges;
  int32_t* overflow;
};

void launch_kmer_prepass(const Reads& R, const pg_window* wins, const int64_t* rlist, int32_t n, int32_t K,
                         long long* out, cudaStream_t s);
// clears full / used / x_ev_fill of the windows in win_list
void launch_kmer_reset(const KmerArgs& a, cudaStream_t s);
// k_kmer_count over the batch's chunks
void launch_kmer_count(const KmerArgs& a, cudaStream_t s);
// k_kmer_exotic over the windows of win_list (after every batch of them was counted)
void launch_kmer_exotic(const KmerArgs& a, cudaStream_t s);
// k_kmer_edges over the batch's windows (windows marked full write none)
void launch_kmer_edges(const KmerArgs& a, cudaStream_t s);

}  // namespace pg
