// pg_kmer.cuh — arguments of the K-mer tally kernels (pg_kmer.cu).
#pragma once
#include "pg_internal.cuh"

namespace pg {

// reads [lo, hi) of window w, walked by one CTA of k_kmer_count
struct KmerChunk {
  int64_t lo, hi;
  int32_t w, pad;
};

struct KmerArgs {
  Reads R;
  const pg_window* windows;
  int32_t win_begin;          // first window of this batch
  int32_t K;
  int32_t min_qual, default_qual, min_depth;
  int32_t wide;               // 1: 128-bit 2-bit keys (K <= 63), 4-word exotic keys, pg_kmer_edge_wide output
  const KmerChunk* chunks;    // the batch's read chunks
  int32_t n_chunks;
  int32_t* full;              // per window: 1 when a probe sequence ran past the bound (count again, larger)
  unsigned long long* used;   // per window: distinct K-mers inserted
  // 2-bit tables: slots [slot_base[w], slot_base[w] + slot_cap[w]) of window w
  const int64_t* slot_base;
  const int64_t* slot_cap;
  unsigned long long* keys;   // kEmpty = free; wide: two words per slot (16-byte aligned)
  uint32_t* cnt;              // 4 per slot
  unsigned long long* qs;     // 4 per slot
  uint32_t* mq_sum;
  uint32_t* q_sum;
  // exotic tables (4-bit keys), single writer per window
  const int64_t* x_base;
  const int64_t* x_cap;
  unsigned long long* x_keys; // 2 per slot (wide: 4)
  uint8_t* x_used;
  uint32_t* x_cnt;
  unsigned long long* x_qs;
  uint32_t* x_mq;
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

void launch_kmer_prepass(const Reads& R, const pg_window* wins, int32_t n, int32_t K, long long* out,
                         cudaStream_t s);
// k_kmer_count over the batch's chunks, then k_kmer_exotic
void launch_kmer_count(const KmerArgs& a, int32_t n_win, cudaStream_t s);
// k_kmer_edges over the batch's windows
void launch_kmer_edges(const KmerArgs& a, int32_t n_win, cudaStream_t s);

}  // namespace pg
