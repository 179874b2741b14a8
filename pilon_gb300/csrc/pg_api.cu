// pg_api.cu — the C ABI of include/pilon_gb300.h: context, device memory,
// the pipeline driver and result transfer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "pg_internal.cuh"
#include "pg_kmer.cuh"
#include "pg_breaks.cuh"
#include "pg_format.cuh"
#include "pg_host_guard.h"

// NVTX range over one entry point (a profiler shows the host side of each call;
// without a tool attached a push/pop costs a few nanoseconds)
namespace {
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
};
}  // namespace

using namespace pg;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

}  // namespace

struct pg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::string open_err;  // why pg_open failed, when it did
  // reference
  DevBuf ref;
  std::vector<int64_t> ref_off, ref_len;
  // reads
  Reads R{};
  bool have_reads = false;
  DevBuf rd[15];
  ReadExtent ext{};
  DevBuf d_ext, rdesc;
  DevBuf ent_off, ent_sums, entries;  // walk entries of the read store
  int64_t n_entries = 0;
  // per-call buffers
  DevBuf regions, walk_tiles, call_tile_region, call_desc, chunks, stats;
  DevBuf rec_count, rec_qsum, rec_i32[10], rec_call, rec_score, rec_indel_len, rec_ins_str, rec_ev_end;
  DevBuf cand_count, cand_off, tile_sums;
  DevBuf events, events_sorted, cands, pool, counters, run_max, chunk_stats, spool, indel_list;
  int64_t event_cap = 0, pool_cap = 0, spool_cap = 0;
  int32_t cand_cap = 0;
  DevBuf staging_dev;
  void* staging_host = nullptr;
  size_t staging_cap = 0;
  // last call
  std::vector<RegionDev> regions_h;
  std::vector<StatsDev> stats_h;
  int32_t n_regions = 0;
  int64_t n_positions = 0;
  bool have_results = false;
  int32_t n_call_tiles = 0;
  // timing
  cudaEvent_t e0 = nullptr, e1 = nullptr, w0 = nullptr, w1 = nullptr;
  std::vector<cudaEvent_t> wev;  // pairs around each walk launch
  int32_t n_runs = 0;
  double walk_ms = 0, total_ms = 0;
  int32_t launches = 0;
  // k-mer tally
  DevBuf kwin, kpre, kslot_base, kslot_cap, kx_base, kx_cap, kslots, kwlist;
  DevBuf kx_keys, kx_used, kx_cnt, kx_qs, kx_q, kedges, kcount, kx_ev, kx_evbase, kx_evcap, kx_evfill;
  DevBuf kwflag, kused, kchunks, klist;
  double tally_ms = 0;  // kernel time of the last tally (CUDA events)
  int64_t tally_events = 0, tally_distinct = 0, tally_max_batch_bytes = 0;
  int32_t tally_batches = 0;
  // VCF formatting
  DevBuf vlen, vsums, vtext, vname;
  // break candidates
  DevBuf bfrag, bsums, btiles, bgaps, bruns, bcnt, boff, bout;
  DevBuf druns, dout, dcount;  // duplication events
  DevBuf chg_count, chg_off, chg_out;  // changes of the last call (pg_fetch_changes)
  int64_t brk_n = -1;             // breaks of the last pileup call on the device, -1: not found yet
  int32_t brk_mmd = 0;
  // CUDA graph of the batched pipeline, replayed while the plan and buffers are unchanged
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  uint64_t graph_key = 0;
  bool graph_valid = false;  // cleared whenever a buffer the graph uses is reallocated
  uint64_t plan_key = 0;     // the plan now in the device buffers (0: none); cleared with graph_valid
  uint64_t ref_gen = 0;      // counts pg_set_reference calls
  int32_t use_graph = 1;
  int32_t graph_replays = 0;
  bool capturing = false;
  // tuning
  int32_t tile_width = 2048, warps = 16, packed = 0;
  uint32_t mode_mq1 = 0;  // most common adjusted mq + 1 of the read store's fast-path reads
};

namespace {

pg_status fail(pg_ctx* c, pg_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return s;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(c, PG_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));        \
  } while (0)

pg_status ensure(pg_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes <= b.cap && b.p) return PG_OK;
  // a captured graph holds the old address: it must not be replayed again
  c->graph_valid = false;
  c->graph_key = 0;
  c->plan_key = 0;  // the plan buffers may be among those reallocated
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  size_t want = std::max<size_t>(bytes + bytes / 4, 256);
  cudaError_t e = cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, PG_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", want, cudaGetErrorString(e));
  }
  b.cap = want;
  return PG_OK;
}

void release(DevBuf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
}

template <class T>
T* P(DevBuf& b) {
  return (T*)b.p;
}

DevParams to_dev(const pg_params* p) {
  // zeroed first: the graph key hashes the whole struct, tail padding included
  DevParams d;
  memset(&d, 0, sizeof d);
  d.min_mq = p->min_mq; d.min_qual = p->min_qual; d.flank = p->flank; d.default_qual = p->default_qual;
  d.min_min_depth = p->min_min_depth; d.nonpf = p->nonpf; d.duplicates = p->duplicates;
  d.old_indel = p->old_indel; d.fix_amb = p->fix_amb; d.long_read = p->long_read; d.bam_type = p->bam_type;
  d.long_read_only = p->long_read_only; d.min_depth = p->min_depth;
  d.huge = 5 * (p->bam_type == PG_BAM_FRAGS ? 500 : 10000);
  return d;
}

Records records(pg_ctx* c) {
  Records r;
  r.count = P<int4>(c->rec_count);
  r.qual_sum = P<longlong2>(c->rec_qsum);
  r.mq_sum = P<int32_t>(c->rec_i32[0]);
  r.q_sum = P<int32_t>(c->rec_i32[1]);
  r.bad_pair = P<int32_t>(c->rec_i32[2]);
  r.clips = P<int32_t>(c->rec_i32[3]);
  r.deletions = P<int32_t>(c->rec_i32[4]);
  r.del_qual = P<int32_t>(c->rec_i32[5]);
  r.insertions = P<int32_t>(c->rec_i32[6]);
  r.ins_qual = P<int32_t>(c->rec_i32[7]);
  r.phys_cov = P<int32_t>(c->rec_i32[8]);
  r.insert_size = P<int32_t>(c->rec_i32[9]);
  r.ev_end = P<int32_t>(c->rec_ev_end);
  r.call = P<uint32_t>(c->rec_call);
  r.score = P<int64_t>(c->rec_score);
  r.indel_len = P<int32_t>(c->rec_indel_len);
  r.ins_str = P<int32_t>(c->rec_ins_str);
  return r;
}

// Counters kept on the device for one call: [0] events, [1] pool bytes,
// [2] string-pool words of the current run, [3] most string-pool words of any run.
enum { CNT_EVENTS = 0, CNT_POOL = 1, CNT_SPOOL = 2, CNT_SPOOL_MAX = 3, CNT_N = 4 };
// run_max: [0] max events of a run, [1] max candidates of a run
__global__ void k_track(unsigned long long* counters, const int32_t* cand_total, unsigned long long* run_max) {
  atomicMax(&run_max[0], counters[CNT_EVENTS]);
  atomicMax(&run_max[1], (unsigned long long)(*cand_total));
  atomicMax(&counters[CNT_SPOOL_MAX], counters[CNT_SPOOL]);
}

struct Plan {
  std::vector<WalkTile> walk;
  std::vector<int32_t> call_region;
  std::vector<ReadChunk> chunks;
};

inline uint64_t fnv(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = (const unsigned char*)p;
  for (size_t k = 0; k < n; k++) h = (h ^ b[k]) * 0x100000001b3ull;
  return h;
}
std::mutex& upload_mutex(int device) {
  static std::mutex m[64];
  return m[(unsigned)device % 64u];
}

// the same over 64-bit words, each mixed before it is folded in
inline uint64_t fnv64(uint64_t h, const int64_t* w, size_t n) {
  for (size_t k = 0; k < n; k++) {
    uint64_t x = (uint64_t)w[k];
    x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33;
    h = (h ^ x) * 0x100000001b3ull;
  }
  return h;
}

}  // namespace

extern "C" {

const char* pg_version(void) { return "pilon_gb300 0.1 (sm_103a)"; }

void pg_default_params(pg_params* p) {
  if (!p) return;
  memset(p, 0, sizeof *p);
  p->min_mq = 0;
  p->min_qual = 0;
  p->flank = 10;
  p->default_qual = 10;
  p->min_min_depth = 5;
  p->min_depth = 0.1;
  p->bam_type = PG_BAM_FRAGS;
}

pg_status pg_open(pg_ctx** out, int device) try {
  if (!out) return PG_ERR_ARG;
  *out = nullptr;
  pg_ctx* c = new pg_ctx();
  c->device = device;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    *out = c;
    fail(c, PG_ERR_CUDA, "no CUDA device %d", device);
    c->open_err = c->err;
    return PG_ERR_CUDA;
  }
  cudaSetDevice(device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    c->stream = nullptr;
    *out = c;
    fail(c, PG_ERR_CUDA, "cudaStreamCreate failed");
    c->open_err = c->err;
    return PG_ERR_CUDA;
  }
  cudaEventCreate(&c->e0);
  cudaEventCreate(&c->e1);
  cudaEventCreate(&c->w0);
  cudaEventCreate(&c->w1);
  *out = c;
  return PG_OK;
} PG_HOST_CATCH(out ? *out : nullptr)

void pg_close(pg_ctx* c) {
  if (!c) return;
  if (c->stream) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
  }
  DevBuf* all[] = {&c->ref, &c->d_ext, &c->rdesc, &c->ent_off, &c->ent_sums, &c->entries, &c->regions, &c->walk_tiles, &c->call_tile_region, &c->call_desc, &c->chunks, &c->stats,
                   &c->rec_count, &c->rec_qsum, &c->rec_call, &c->rec_score, &c->rec_indel_len, &c->rec_ins_str,
                   &c->rec_ev_end, &c->cand_count, &c->cand_off, &c->tile_sums,
                   &c->events, &c->events_sorted, &c->cands, &c->pool, &c->counters, &c->run_max, &c->staging_dev,
                   &c->chunk_stats, &c->spool, &c->indel_list};
  for (DevBuf* b : all) release(*b);
  DevBuf* km[] = {&c->kwin, &c->kpre, &c->kslot_base, &c->kslot_cap, &c->kx_base, &c->kx_cap, &c->kslots, &c->kwlist,
                  &c->kx_keys, &c->kx_used, &c->kx_cnt, &c->kx_qs, &c->kx_q,
                  &c->kedges, &c->kcount, &c->kx_ev, &c->kx_evbase, &c->kx_evcap, &c->kx_evfill, &c->kwflag,
                  &c->kused, &c->kchunks, &c->klist, &c->vlen,
                  &c->vsums, &c->vtext, &c->vname, &c->bfrag, &c->bsums, &c->btiles, &c->bgaps, &c->bruns,
                  &c->bcnt, &c->boff, &c->bout, &c->druns, &c->dout, &c->dcount, &c->chg_count, &c->chg_off,
                  &c->chg_out};
  for (DevBuf* b : km) release(*b);
  for (auto& b : c->rec_i32) release(b);
  for (auto& b : c->rd) release(b);
  if (c->staging_host) cudaFreeHost(c->staging_host);
  if (c->e0) cudaEventDestroy(c->e0);
  if (c->e1) cudaEventDestroy(c->e1);
  if (c->w0) cudaEventDestroy(c->w0);
  if (c->w1) cudaEventDestroy(c->w1);
  for (cudaEvent_t e : c->wev) cudaEventDestroy(e);
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* pg_last_error(const pg_ctx* c) { return c ? c->err.c_str() : "null context"; }

pg_status pg_set_tuning(pg_ctx* c, int32_t tile_width, int32_t warps_per_cta, int32_t variant) try {
  if (!c) return PG_ERR_ARG;
  if (tile_width) {
    if (tile_width < 256 || tile_width > 4096 || (tile_width & (tile_width - 1)))
      return fail(c, PG_ERR_ARG, "tile width %d must be a power of two in [256, 4096]", tile_width);
    c->tile_width = tile_width;
  }
  if (warps_per_cta) {
    if (warps_per_cta < 1 || warps_per_cta > 16) return fail(c, PG_ERR_ARG, "warps per CTA must be in [1, 16]");
    c->warps = warps_per_cta;
  }
  if (variant >= 0) {
    if (variant > 3) return fail(c, PG_ERR_ARG, "variant must be 0, 1, 2 or 3");
    c->packed = variant;
  }
  return PG_OK;
} PG_HOST_CATCH(c)

// Pilon's --defaultqual is a Byte (S/Pilon.scala:53, 144: value.toByte throws
// outside -128..127); the walk's packed counters rely on that range too.
static pg_status check_default_qual(pg_ctx* c, const pg_params* p) {
  if (p->default_qual < -128 || p->default_qual > 127)
    return fail(c, PG_ERR_ARG, "default_qual %d is outside a byte (-128..127)", p->default_qual);
  return PG_OK;
}

// A context whose pg_open failed has no stream; calls that would use the
// device on it fail with PG_ERR_STATE instead of running on the legacy stream.
static pg_status not_open(pg_ctx* c) {
  return fail(c, PG_ERR_STATE, "the context is not open (pg_open failed: %s)", c->open_err.c_str());
}

pg_status pg_sync(pg_ctx* c) try {
  if (!c) return PG_ERR_ARG;
  if (!c->stream) return not_open(c);
  cudaSetDevice(c->device);
  CK(cudaStreamSynchronize(c->stream));
  return PG_OK;
} PG_HOST_CATCH(c)

pg_status pg_set_reference(pg_ctx* c, int32_t n, const int64_t* lens, const uint8_t* const* bases) try {
  const Range nvtx_range("pg_set_reference");
  if (!c || n < 0 || (n > 0 && (!lens || !bases))) return fail(c, PG_ERR_ARG, "bad reference arguments");
  for (int i = 0; i < n; i++) {
    if (lens[i] < 0 || (lens[i] > 0 && !bases[i])) return fail(c, PG_ERR_ARG, "contig %d has no bases", i);
    // positions are 32-bit, as Pilon's (Scala Int; a contig is one JVM byte array)
    if (lens[i] > INT32_MAX) return fail(c, PG_ERR_ARG, "contig %d is longer than 2^31 - 1 bases", i);
  }
  if (!c->stream) return not_open(c);
  cudaSetDevice(c->device);
  c->ref_gen++;  // region offsets into the reference change: the next plan is uploaded again
  c->plan_key = 0;
  c->ref_off.assign(n, 0);
  c->ref_len.assign(lens, lens + n);
  int64_t total = 0;
  for (int i = 0; i < n; i++) {
    c->ref_off[i] = total;
    total += lens[i];
  }
  // 16 bytes of slack: k_call stages the aligned word that holds a reference byte
  pg_status s = ensure(c, c->ref, (size_t)std::max<int64_t>(total, 1) + 16);
  if (s) return s;
  for (int i = 0; i < n; i++)
    if (lens[i] > 0)
      CK(cudaMemcpyAsync(P<uint8_t>(c->ref) + c->ref_off[i], bases[i], lens[i], cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return PG_OK;
} PG_HOST_CATCH(c)

static pg_status finish_reads(pg_ctx* c) {
  c->have_reads = false;
  pg_status s = ensure(c, c->d_ext, sizeof(ReadExtent));
  if (s) return s;
  s = ensure(c, c->rdesc, (size_t)std::max<int64_t>(c->R.n, 1) * 2 * sizeof(int4));
  if (s) return s;
  c->R.desc = P<int4>(c->rdesc);
  launch_read_extent(c->R, P<ReadExtent>(c->d_ext), P<int4>(c->rdesc), c->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(&c->ext, c->d_ext.p, sizeof(ReadExtent), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (c->ext.bad_read)
    return fail(c, PG_ERR_ARG, "read %llu: CIGAR, base or quality offsets leave their arrays",
                (unsigned long long)c->ext.bad_read - 1);
  if (c->ext.unsorted) return fail(c, PG_ERR_ARG, "reads are not sorted by position within each reference");
  // the walk entries (one per M/=/X or S operator), made once per read store
  const int64_t n = c->R.n;
  if ((s = ensure(c, c->ent_off, 8 * (size_t)(n + 1)))) return s;
  if ((s = ensure(c, c->ent_sums, 8 * (size_t)((n + 1 + 1023) / 1024 + 2)))) return s;
  c->R.entry_off = P<int64_t>(c->ent_off);
  launch_entry_count(c->R, P<int64_t>(c->ent_off), P<int64_t>(c->ent_sums), c->stream);
  CK(cudaGetLastError());
  int64_t total = 0;
  CK(cudaMemcpyAsync(&total, P<int64_t>(c->ent_off) + n, 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if ((s = ensure(c, c->entries, 48 * (size_t)std::max<int64_t>(total, 1)))) return s;
  c->R.entries = P<int4>(c->entries);
  c->n_entries = total;
  launch_entry_fill(c->R, P<int64_t>(c->ent_off), P<int4>(c->entries), c->stream);
  CK(cudaGetLastError());
  c->mode_mq1 = 0;
  for (uint32_t b = 1, best = 0; b <= 256; b++)
    if (c->ext.mq1_hist[b] > best) { best = c->ext.mq1_hist[b]; c->mode_mq1 = b; }
  c->have_reads = true;
  c->have_results = false;
  return PG_OK;
}

static pg_status upload_reads(pg_ctx* c, const pg_reads* h, bool packed);

pg_status pg_set_reads(pg_ctx* c, const pg_reads* h) try {
  const Range nvtx_range("pg_set_reads");
  return upload_reads(c, h, false);
} PG_HOST_CATCH(c)

pg_status pg_set_reads_packed(pg_ctx* c, const pg_reads* h) try {
  const Range nvtx_range("pg_set_reads_packed");
  return upload_reads(c, h, true);
} PG_HOST_CATCH(c)

// packed: the offsets and alignment ends are not read from the host (they may
// be NULL); the device derives them from the lengths and the CIGARs
static pg_status upload_reads(pg_ctx* c, const pg_reads* h, bool packed) {
  if (!c || !h || h->n_reads < 0) return fail(c, PG_ERR_ARG, "bad reads");
  // the store is replaced from here on: until it is complete and checked no
  // call may use it (a failed upload leaves the context without reads)
  c->have_reads = false;
  c->have_results = false;
  if (h->n_cigar_words < 0 || h->seq_bytes < 0 || h->qual_bytes < 0)
    return fail(c, PG_ERR_ARG, "negative array length in the read store");
  if (!c->stream) return not_open(c);
  cudaSetDevice(c->device);
  const int64_t n = h->n_reads;
  const void* src[15] = {h->pos, h->aend, h->tlen, h->ref_id, h->mate_ref_id, h->l_seq, h->flag, h->n_cigar,
                         h->mapq, h->seq, h->qual, h->cigar_off, h->seq_off, h->qual_off, h->cigar};
  const size_t bytes[15] = {(size_t)n * 4, (size_t)n * 4, (size_t)n * 4, (size_t)n * 4, (size_t)n * 4,
                            (size_t)n * 4, (size_t)n * 2, (size_t)n * 2, (size_t)n,
                            (size_t)h->seq_bytes, (size_t)h->qual_bytes, (size_t)n * 8, (size_t)n * 8,
                            (size_t)n * 8, (size_t)h->n_cigar_words * 4};
  // fields the packed upload derives on the device: aend (1) and the three offsets (11-13)
  auto derived = [&](int k) { return packed && (k == 1 || k == 11 || k == 12 || k == 13); };
  for (int k = 0; k < 15; k++) {
    if (bytes[k] && !src[k] && !derived(k)) return fail(c, PG_ERR_ARG, "reads field %d is null", k);
    pg_status s = ensure(c, c->rd[k], std::max<size_t>(bytes[k], 16));
    if (s) return s;
  }
  {
    // Uploads to one device take turns: the host link is saturated by one
    // upload (about 210 GB/s on a GB300 whatever the number of streams), so two
    // contexts uploading at once only split it and then compute at once; in
    // turns, one context's upload overlaps the other's kernels.  The context's
    // earlier work is waited for before the turn is taken.
    CK(cudaStreamSynchronize(c->stream));
    std::lock_guard<std::mutex> turn(upload_mutex(c->device));
    for (int k = 0; k < 15; k++)
      if (bytes[k] && !derived(k))
        CK(cudaMemcpyAsync(c->rd[k].p, src[k], bytes[k], cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  Reads& R = c->R;
  R.n = n;
  R.pos = P<int32_t>(c->rd[0]); R.aend = P<int32_t>(c->rd[1]); R.tlen = P<int32_t>(c->rd[2]);
  R.ref_id = P<int32_t>(c->rd[3]); R.mate_ref_id = P<int32_t>(c->rd[4]); R.l_seq = P<int32_t>(c->rd[5]);
  R.flag = P<uint16_t>(c->rd[6]); R.n_cigar = P<uint16_t>(c->rd[7]); R.mapq = P<uint8_t>(c->rd[8]);
  R.seq = P<uint8_t>(c->rd[9]); R.qual = P<uint8_t>(c->rd[10]); R.cigar_off = P<int64_t>(c->rd[11]);
  R.seq_off = P<int64_t>(c->rd[12]); R.qual_off = P<int64_t>(c->rd[13]); R.cigar = P<uint32_t>(c->rd[14]);
  R.n_cigar_words = h->n_cigar_words; R.seq_bytes = h->seq_bytes; R.qual_bytes = h->qual_bytes;
  if (packed && n > 0) {
    const int32_t nb = (int32_t)((n + 1023) / 1024);
    pg_status s = ensure(c, c->ent_sums, 8 * (size_t)(nb + 2));
    if (s) return s;
    launch_packed_lengths(R, P<int64_t>(c->rd[11]), P<int64_t>(c->rd[12]), P<int64_t>(c->rd[13]), c->stream);
    int64_t totals[3] = {0, 0, 0};
    for (int k = 0; k < 3; k++) {  // exclusive scans: the offsets; the totals must be the arrays' lengths
      launch_scan64(P<int64_t>(c->rd[11 + k]), n, P<int64_t>(c->ent_sums), c->stream);
      CK(cudaMemcpyAsync(&totals[k], P<int64_t>(c->ent_sums) + nb, 8, cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
    }
    if (totals[0] != h->n_cigar_words || totals[1] != h->seq_bytes || totals[2] != h->qual_bytes)
      return fail(c, PG_ERR_ARG, "packed read store: the reads' CIGAR words, bases or qualities do not fill "
                  "their arrays (%lld / %lld / %lld against %lld / %lld / %lld)", (long long)totals[0],
                  (long long)totals[1], (long long)totals[2], (long long)h->n_cigar_words,
                  (long long)h->seq_bytes, (long long)h->qual_bytes);
    launch_packed_aend(R, P<int32_t>(c->rd[1]), c->stream);
    CK(cudaGetLastError());
  }
  return finish_reads(c);
}

pg_status pg_set_reads_device(pg_ctx* c, const pg_reads* d) try {
  const Range nvtx_range("pg_set_reads_device");
  if (!c || !d || d->n_reads < 0) return fail(c, PG_ERR_ARG, "bad reads");
  if (d->n_cigar_words < 0 || d->seq_bytes < 0 || d->qual_bytes < 0)
    return fail(c, PG_ERR_ARG, "negative array length in the read store");
  if (!c->stream) return not_open(c);
  cudaSetDevice(c->device);
  Reads& R = c->R;
  R.n = d->n_reads;
  R.pos = d->pos; R.aend = d->aend; R.tlen = d->tlen; R.ref_id = d->ref_id; R.mate_ref_id = d->mate_ref_id;
  R.l_seq = d->l_seq; R.flag = d->flag; R.n_cigar = d->n_cigar; R.mapq = d->mapq; R.seq = d->seq;
  R.qual = d->qual; R.cigar_off = d->cigar_off; R.seq_off = d->seq_off; R.qual_off = d->qual_off;
  R.cigar = d->cigar;
  R.n_cigar_words = d->n_cigar_words; R.seq_bytes = d->seq_bytes; R.qual_bytes = d->qual_bytes;
  return finish_reads(c);
} PG_HOST_CATCH(c)

static pg_status stage(pg_ctx* c, size_t bytes) {
  if (bytes <= c->staging_cap) return PG_OK;
  c->graph_valid = false;
  c->graph_key = 0;
  c->plan_key = 0;
  if (c->staging_host) cudaFreeHost(c->staging_host);
  c->staging_host = nullptr;
  size_t want = bytes + bytes / 4 + 4096;
  if (cudaMallocHost(&c->staging_host, want) != cudaSuccess) {
    c->staging_cap = 0;
    cudaGetLastError();
    return fail(c, PG_ERR_NOMEM, "cudaMallocHost of %zu bytes failed", want);
  }
  c->staging_cap = want;
  return ensure(c, c->staging_dev, want);
}

// Runs the pipeline for regions [r0, r1) (tiles and chunks of those regions).
static void run_range(pg_ctx* c, const Plan& plan, int32_t r0, int32_t r1, const DevParams& dp) {
  cudaStream_t s = c->stream;
  const RegionDev& a = c->regions_h[r0];
  const RegionDev& b = c->regions_h[r1 - 1];
  const int32_t w0 = a.walk_tile0, wn = b.walk_tile0 + b.n_walk_tiles - w0;
  const int32_t t0 = a.call_tile0, tn = b.call_tile0 + b.n_call_tiles - t0;
  int32_t ch0 = -1, chn = 0;
  for (int32_t k = 0; k < (int32_t)plan.chunks.size(); k++) {  // chunks are in region order
    if (plan.chunks[k].region >= r0 && plan.chunks[k].region < r1) {
      if (ch0 < 0) ch0 = k;
      chn++;
    }
  }
  if (ch0 < 0) ch0 = 0;
  RegionDev* d_regions = P<RegionDev>(c->regions);
  StatsDev* d_stats = P<StatsDev>(c->stats);
  Records rec = records(c);
  unsigned long long* counters = P<unsigned long long>(c->counters);

  cudaMemsetAsync(P<int32_t>(c->cand_count) + t0, 0, sizeof(int32_t) * (tn + 1), s);
  cudaMemsetAsync(&counters[CNT_EVENTS], 0, sizeof(unsigned long long), s);
  cudaMemsetAsync(&counters[CNT_SPOOL], 0, sizeof(unsigned long long), s);

  launch_tile_ranges(c->R, d_regions, P<WalkTile>(c->walk_tiles) + w0, wn, P<ReadExtent>(c->d_ext), d_stats, s);

  WalkArgs wa;
  wa.R = c->R; wa.regions = d_regions; wa.tiles = P<WalkTile>(c->walk_tiles); wa.n_tiles = wn;
  wa.rec = rec; wa.stats = d_stats; wa.P = dp; wa.ref = P<uint8_t>(c->ref); wa.tile_width = c->tile_width;
  wa.packed = c->packed;
  wa.mode_mq1 = c->mode_mq1;
  wa.reads_per_pass = walk_reads_per_pass(dp.default_qual);
  while ((int32_t)c->wev.size() < 2 * (c->n_runs + 1)) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    c->wev.push_back(e);
  }
  // inside a stream capture the records must be external to become event nodes of the graph
  const unsigned evf = c->capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  cudaEventRecordWithFlags(c->wev[2 * c->n_runs], s, evf);
  launch_walk(wa, w0, wn, c->warps, s);
  cudaEventRecordWithFlags(c->wev[2 * c->n_runs + 1], s, evf);
  c->n_runs++;

  EventArgs ea;
  ea.R = c->R; ea.regions = d_regions; ea.chunks = P<ReadChunk>(c->chunks); ea.n_chunks = chn; ea.rec = rec;
  ea.stats = d_stats; ea.P = dp; ea.ref = P<uint8_t>(c->ref); ea.events = P<Event>(c->events);
  ea.n_events = &counters[CNT_EVENTS]; ea.event_cap = c->event_cap;
  ea.chunk_stats = P<ChunkStats>(c->chunk_stats);
  ea.spool = P<uint64_t>(c->spool); ea.spool_fill = &counters[CNT_SPOOL]; ea.spool_cap = c->spool_cap;
  ea.indel_list = P<int64_t>(c->indel_list);
  launch_read_events(ea, ch0, chn, s);

  int32_t max_chunks = 0;
  for (int32_t r = r0; r < r1; r++) max_chunks = std::max(max_chunks, c->regions_h[r].n_chunks);
  launch_region_prep(d_regions + r0, d_stats + r0, P<ChunkStats>(c->chunk_stats), r1 - r0, max_chunks, dp, s);
  // the tiles' sums, their segmented prefixes, then the scan's block sums (3 words per 1024 tiles)
  {
    int32_t* ts = P<int32_t>(c->tile_sums);
    const int64_t w = 3 * ((int64_t)c->n_call_tiles + 1);
    launch_physcov_scan(d_regions, P<int32_t>(c->call_tile_region), t0, tn, rec, d_stats, ts, ts + w, ts + 2 * w,
                        r0, r1 - r0, s);
  }
  launch_event_scatter(P<Event>(c->events), &counters[CNT_EVENTS], rec.ev_end, P<Event>(c->events_sorted), s,
                       c->event_cap);

  CallArgs ca;
  ca.R = c->R; ca.regions = d_regions; ca.call_tile_region = P<int32_t>(c->call_tile_region);
  ca.call_desc = P<CallDesc>(c->call_desc);
  ca.n_call_tiles = tn; ca.rec = rec; ca.stats = d_stats; ca.P = dp; ca.ref = P<uint8_t>(c->ref);
  ca.ev_sorted = P<Event>(c->events_sorted);
  ca.event_cap = c->event_cap;
  ca.spool = P<uint64_t>(c->spool);
  ca.cand_count = P<int32_t>(c->cand_count); ca.pool = P<char>(c->pool); ca.pool_fill = &counters[CNT_POOL];
  ca.pool_cap = c->pool_cap;
  launch_call(ca, t0, tn, s);
  launch_scan_small(P<int32_t>(c->cand_count) + t0, P<int32_t>(c->cand_off) + t0, tn, s);
  launch_cand_list(ca, P<int32_t>(c->cand_off), P<Cand>(c->cands), c->cand_cap, t0, tn, s);
  launch_resolve(d_regions + r0, r1 - r0, P<int32_t>(c->cand_off), P<Cand>(c->cands), c->cand_cap, d_stats + r0, s);
  launch_apply_spans(ca, P<Cand>(c->cands), P<int32_t>(c->cand_off) + t0 + tn, c->cand_cap, s);
  k_track<<<1, 1, 0, s>>>(counters, P<int32_t>(c->cand_off) + t0 + tn, P<unsigned long long>(c->run_max));
  // kernels of this run: tile ranges + walk, read events, region prep, three
  // scan phases, event scatter, call descriptors, call, candidate scan,
  // candidate list, resolve, span update, overflow tracking
  // kernels of this call: tile ranges and walk; read events and indels; region prep; the five scan
  // phases; event scatter; call descriptors and calls; the candidate count scan and list; resolve;
  // spans; k_track
  c->launches += 2 * (wn > 0) + 2 * (chn > 0) + 1 + 5 * (tn > 0) + (c->event_cap > 0) + 2 * (tn > 0) + 1 +
                 (tn > 0) + 1 + (c->cand_cap > 0) + 1;
}

pg_status pg_pileup_regions(pg_ctx* c, const pg_region* regs, int32_t n_regions, const pg_params* params,
                            int32_t batched) try {
  const Range nvtx_range("pg_pileup_regions");
  if (!c || (n_regions > 0 && !regs) || !params || n_regions < 0) return fail(c, PG_ERR_ARG, "bad arguments");
  if (params->min_qual < 0 || params->flank < 0 || params->min_mq < 0)
    return fail(c, PG_ERR_ARG, "min_qual, min_mq and flank must be >= 0");
  if (pg_status s0 = check_default_qual(c, params)) return s0;
  if (!c->have_reads) return fail(c, PG_ERR_STATE, "pg_set_reads must come first");
  cudaSetDevice(c->device);
  c->brk_n = -1;
  c->have_results = false;
  const int T = c->tile_width;
  // ---- plan
  Plan plan;
  c->regions_h.resize(n_regions);
  int64_t pos = 0;
  for (int32_t r = 0; r < n_regions; r++) {
    const pg_region& q = regs[r];
    if (q.contig < 0 || q.contig >= (int32_t)c->ref_len.size())
      return fail(c, PG_ERR_ARG, "region %d: contig %d out of range", r, q.contig);
    const int64_t clen = c->ref_len[q.contig];
    if (q.start < 1 || q.stop < q.start || q.stop > clen)
      return fail(c, PG_ERR_ARG, "region %d: [%d, %d] outside contig of length %lld", r, q.start, q.stop,
                  (long long)clen);
    if (q.read_begin < 0 || q.read_end < q.read_begin || q.read_end > c->R.n)
      return fail(c, PG_ERR_ARG, "region %d: read range out of bounds", r);
    RegionDev& g = c->regions_h[r];
    g.contig = q.contig; g.start = q.start; g.stop = q.stop; g.size = q.stop - q.start + 1;
    g.pos_base = pos; g.ref_off = c->ref_off[q.contig]; g.contig_len = clen;
    g.read_begin = q.read_begin; g.read_end = q.read_end;
    g.qs = (int32_t)std::max<int64_t>((int64_t)q.start - 10000, 0);
    g.qe = (int32_t)std::min<int64_t>((int64_t)q.stop + 10000, clen);
    g.walk_tile0 = (int32_t)plan.walk.size();
    g.n_walk_tiles = (g.size + T - 1) / T;
    for (int32_t k = 0; k < g.n_walk_tiles; k++)
      plan.walk.push_back(WalkTile{r, k * T, std::min(T, g.size - k * T), 0, 0, 0});
    g.call_tile0 = (int32_t)plan.call_region.size();
    g.n_call_tiles = (g.size + kCallTile - 1) / kCallTile;
    for (int32_t k = 0; k < g.n_call_tiles; k++) plan.call_region.push_back(r);
    g.chunk0 = (int32_t)plan.chunks.size();
    for (int64_t lo = q.read_begin; lo < q.read_end; lo += kReadsPerChunk)
      plan.chunks.push_back(ReadChunk{r, 0, lo, std::min<int64_t>(lo + kReadsPerChunk, q.read_end)});
    g.n_chunks = (int32_t)plan.chunks.size() - g.chunk0;
    pos += g.size;
  }
  c->n_regions = n_regions;
  c->n_positions = pos;
  const int32_t n_call = (int32_t)plan.call_region.size();
  c->n_call_tiles = n_call;
  if (n_regions == 0) {
    c->have_results = true;
    return PG_OK;
  }
  // ---- buffers
  pg_status s;
#define EN(buf, bytes) \
  if ((s = ensure(c, buf, (bytes)))) return s;
  EN(c->regions, sizeof(RegionDev) * n_regions);
  EN(c->stats, sizeof(StatsDev) * n_regions);
  EN(c->walk_tiles, sizeof(WalkTile) * std::max<size_t>(plan.walk.size(), 1));
  EN(c->call_tile_region, sizeof(int32_t) * (n_call + 1));
  EN(c->call_desc, sizeof(CallDesc) * (n_call + 1));
  EN(c->chunks, sizeof(ReadChunk) * std::max<size_t>(plan.chunks.size(), 1));
  EN(c->chunk_stats, sizeof(ChunkStats) * std::max<size_t>(plan.chunks.size(), 1));
  EN(c->indel_list, sizeof(int64_t) * kReadsPerChunk * std::max<size_t>(plan.chunks.size(), 1));
  EN(c->rec_count, 16 * (size_t)pos);
  EN(c->rec_qsum, 32 * (size_t)pos);
  for (auto& b : c->rec_i32) EN(b, 4 * (size_t)pos);
  EN(c->rec_call, 4 * (size_t)pos);
  EN(c->rec_score, 8 * (size_t)pos);
  EN(c->rec_indel_len, 4 * (size_t)pos);
  EN(c->rec_ins_str, 4 * (size_t)pos);
  EN(c->rec_ev_end, 4 * (size_t)pos);
  for (DevBuf* b : {&c->cand_count, &c->cand_off}) EN(*b, sizeof(int32_t) * (n_call + 2));
  EN(c->tile_sums, sizeof(int32_t) * 3 * (2 * (n_call + 1) + (n_call / 1024 + 2)));
  EN(c->counters, sizeof(unsigned long long) * CNT_N);
  EN(c->run_max, sizeof(unsigned long long) * 2);
  if (c->event_cap == 0) c->event_cap = (int64_t)(2 * c->ext.n_indel_ops + 4096);
  if (c->cand_cap == 0) c->cand_cap = (int32_t)std::min<int64_t>(pos / 16 + 4096, INT32_MAX / 2);
  if (c->pool_cap == 0) c->pool_cap = 1 << 20;
  if (c->spool_cap == 0) c->spool_cap = 1 << 16;
  // ---- upload the plan
  const size_t b_reg = sizeof(RegionDev) * n_regions, b_walk = sizeof(WalkTile) * plan.walk.size(),
               b_call = sizeof(int32_t) * n_call, b_ch = sizeof(ReadChunk) * plan.chunks.size();
  if ((s = stage(c, b_reg + b_walk + b_call + b_ch + 64))) return s;
  {
    char* h = (char*)c->staging_host;
    memcpy(h, c->regions_h.data(), b_reg);
    memcpy(h + b_reg, plan.walk.data(), b_walk);
    memcpy(h + b_reg + b_walk, plan.call_region.data(), b_call);
    memcpy(h + b_reg + b_walk + b_call, plan.chunks.data(), b_ch);
  }
  const DevParams dp = to_dev(params);
  for (int attempt = 0; attempt < 4; attempt++) {
    if ((s = ensure(c, c->events, sizeof(Event) * c->event_cap))) return s;
    if ((s = ensure(c, c->events_sorted, sizeof(Event) * c->event_cap))) return s;
    if ((s = ensure(c, c->cands, sizeof(Cand) * (size_t)c->cand_cap))) return s;
    if ((s = ensure(c, c->pool, (size_t)c->pool_cap))) return s;
    if ((s = ensure(c, c->spool, 8 * (size_t)c->spool_cap))) return s;
    cudaStream_t st = c->stream;
    // identity of everything the recorded launches depend on.  The plan itself
    // reaches the device through the graph's copy nodes, which read the staging
    // buffer when they run; the launches depend on the regions asked for (their
    // fields, not their padding), the plan's sizes, the parameters, the shape
    // and the buffers.  (Hashing the staged plan byte by byte took 10 ms per
    // call on 3,000 regions.)
    uint64_t key = 0xcbf29ce484222325ull;
    for (int32_t r = 0; r < n_regions; r++) {
      const int64_t f[5] = {regs[r].contig, regs[r].start, regs[r].stop, regs[r].read_begin, regs[r].read_end};
      key = fnv64(key, f, 5);
    }
    const int64_t sizes[7] = {n_regions, (int64_t)b_reg, (int64_t)b_walk, (int64_t)b_call, (int64_t)b_ch,
                              (int64_t)c->tile_width, (int64_t)c->ref_gen};
    key = fnv64(key, sizes, 7);
    // the plan is a function of the regions asked for, the tile width and the
    // reference: copied to the device only when it differs from the one there
    // (outside the recorded graph, so a replay does not queue host-to-device
    // copies behind another context's upload)
    const uint64_t plan_key = key | 1ull;
    if (c->plan_key != plan_key) {
      CK(cudaMemcpyAsync(c->regions.p, c->staging_host, b_reg, cudaMemcpyHostToDevice, st));
      if (b_walk) CK(cudaMemcpyAsync(c->walk_tiles.p, (char*)c->staging_host + b_reg, b_walk, cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(c->call_tile_region.p, (char*)c->staging_host + b_reg + b_walk, b_call,
                         cudaMemcpyHostToDevice, st));
      if (b_ch) CK(cudaMemcpyAsync(c->chunks.p, (char*)c->staging_host + b_reg + b_walk + b_call, b_ch,
                                   cudaMemcpyHostToDevice, st));
      c->plan_key = plan_key;
    }
    key = fnv(key, &dp, sizeof dp);
    key = fnv(key, &c->R, sizeof c->R);
    // every buffer the recorded launches and copies read or write, host staging included
    const void* ptrs[] = {c->ref.p, c->events.p, c->events_sorted.p, c->cands.p, c->pool.p, c->spool.p,
                          c->rec_count.p, c->rec_qsum.p, c->rec_call.p, c->rec_score.p, c->rec_indel_len.p,
                          c->rec_ins_str.p, c->rec_ev_end.p, c->chunk_stats.p, c->stats.p, c->tile_sums.p,
                          c->regions.p, c->walk_tiles.p, c->call_tile_region.p, c->call_desc.p, c->chunks.p,
                          c->cand_count.p,
                          c->cand_off.p, c->indel_list.p, c->counters.p, c->run_max.p, c->d_ext.p, c->rdesc.p,
                          c->staging_host};
    key = fnv(key, ptrs, sizeof ptrs);
    for (auto& b : c->rec_i32) key = fnv(key, &b.p, sizeof b.p);
    const int32_t shape[7] = {c->tile_width, c->warps, c->packed, batched, (int32_t)c->event_cap, c->cand_cap,
                              (int32_t)c->mode_mq1};
    key = fnv(key, shape, sizeof shape);
    key = fnv(key, &c->pool_cap, sizeof c->pool_cap);
    key = fnv(key, &c->spool_cap, sizeof c->spool_cap);
    const bool replay = c->use_graph && batched && c->graph_exec && c->graph_valid && key == c->graph_key;
    const bool capture = c->use_graph && batched && !replay && attempt == 0 && c->graph_key == key + 1;
    c->walk_ms = 0;
    CK(cudaEventRecord(c->e0, st));
    if (replay) {
      CK(cudaGraphLaunch(c->graph_exec, st));
      c->graph_replays++;
    } else {
      if (capture) CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      c->capturing = capture;
      c->launches = 0;
      c->n_runs = 0;
      cudaMemsetAsync(c->stats.p, 0, sizeof(StatsDev) * n_regions, st);
      cudaMemsetAsync(c->counters.p, 0, sizeof(unsigned long long) * CNT_N, st);
      cudaMemsetAsync(c->run_max.p, 0, sizeof(unsigned long long) * 2, st);
      if (batched || n_regions == 1) {
        run_range(c, plan, 0, n_regions, dp);
      } else {
        for (int32_t r = 0; r < n_regions; r++) run_range(c, plan, r, r + 1, dp);
      }
      c->capturing = false;
      if (capture) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (e != cudaSuccess || !g) return fail(c, PG_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(e));
        if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
        if (c->graph) cudaGraphDestroy(c->graph);
        c->graph = g;
        c->graph_exec = nullptr;
        CK(cudaGraphInstantiate(&c->graph_exec, g, 0));
        CK(cudaGraphLaunch(c->graph_exec, st));
        c->graph_key = key;
        c->graph_valid = true;
      } else if (batched && c->use_graph && attempt == 0 && !replay) {
        c->graph_key = key + 1;  // the next identical call records the graph
      }
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(c->e1, st));
    c->stats_h.resize(n_regions);
    unsigned long long hc[CNT_N], hm[2];
    CK(cudaMemcpyAsync(c->stats_h.data(), c->stats.p, sizeof(StatsDev) * n_regions, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hc, c->counters.p, sizeof hc, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hm, c->run_max.p, sizeof hm, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->e0, c->e1));
    c->total_ms = ms;
    c->walk_ms = 0;
    for (int32_t k = 0; k < c->n_runs; k++) {
      CK(cudaEventElapsedTime(&ms, c->wev[2 * k], c->wev[2 * k + 1]));
      c->walk_ms += ms;
    }
    bool grow = false;
    if ((int64_t)hm[0] > c->event_cap) { c->event_cap = (int64_t)hm[0] * 2 + 4096; grow = true; }
    if ((int64_t)hm[1] > c->cand_cap) { c->cand_cap = (int32_t)std::min<int64_t>((int64_t)hm[1] * 2 + 4096, INT32_MAX / 2); grow = true; }
    if ((int64_t)hc[CNT_POOL] > c->pool_cap) { c->pool_cap = (int64_t)hc[CNT_POOL] * 2 + 4096; grow = true; }
    if ((int64_t)hc[CNT_SPOOL_MAX] > c->spool_cap) { c->spool_cap = (int64_t)hc[CNT_SPOOL_MAX] * 2 + 4096; grow = true; }
    if (!grow) {
      for (int32_t r = 0; r < n_regions; r++)
        if (c->stats_h[r].range_error)
          return fail(c, PG_ERR_ARG, "region %d: its read range [%lld, %lld) holds reads of another reference "
                      "(a range must hold the region contig's reads only, in position order)", r,
                      (long long)regs[r].read_begin, (long long)regs[r].read_end);
      c->have_results = true;  // regions without an error keep valid results
      for (int32_t r = 0; r < n_regions; r++)
        if (c->stats_h[r].error)
          return fail(c, PG_ERR_INDEX, "region %d: an indel left shift left the region (the reference throws "
                      "ArrayIndexOutOfBoundsException here); pg_region_stats.error marks every such region", r);
      return PG_OK;
    }
  }
  return fail(c, PG_ERR_LIMIT, "event/candidate buffers kept overflowing");
} PG_HOST_CATCH(c)

pg_status pg_fetch_stats(pg_ctx* c, int32_t r, pg_region_stats* out) try {
  if (!c || !out) return PG_ERR_ARG;
  if (!c->have_results) return fail(c, PG_ERR_STATE, "no results: run pg_pileup_regions first");
  if (r < 0 || r >= c->n_regions) return fail(c, PG_ERR_ARG, "region %d out of range", r);
  const StatsDev& s = c->stats_h[r];
  memset(out, 0, sizeof *out);
  out->base_count = (int64_t)s.base_count;
  out->read_count = (int64_t)s.read_count;
  out->phys_cov_start = s.phys_cov_start;
  out->insert_size_start = s.insert_size_start;
  out->min_depth = s.min_depth;
  out->n_changes = s.n_changes;
  out->fr_count = (int64_t)s.fr_count; out->fr_sum = (int64_t)s.fr_sum; out->fr_sumsq = (int64_t)s.fr_sumsq;
  out->rf_count = (int64_t)s.rf_count; out->rf_sum = (int64_t)s.rf_sum; out->rf_sumsq = (int64_t)s.rf_sumsq;
  out->error = s.error;
  out->n_ins_strings = 0;
  return PG_OK;
} PG_HOST_CATCH(c)

// Copies positions [b, b + n) of every non-null array of o, then the
// insertion characters; one synchronisation.
static pg_status fetch_positions(pg_ctx* c, int64_t b, size_t n, pg_region_out* o) {
  cudaStream_t s = c->stream;
  Records rc = records(c);
  auto cp = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    if (!dst) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
  };
  CK(cp(o->count, rc.count + b, 16 * n));
  CK(cp(o->qual_sum, rc.qual_sum + 2 * b, 32 * n));
  CK(cp(o->mq_sum, rc.mq_sum + b, 4 * n));
  CK(cp(o->q_sum, rc.q_sum + b, 4 * n));
  CK(cp(o->phys_cov, rc.phys_cov + b, 4 * n));
  CK(cp(o->insert_size, rc.insert_size + b, 4 * n));
  CK(cp(o->bad_pair, rc.bad_pair + b, 4 * n));
  CK(cp(o->deletions, rc.deletions + b, 4 * n));
  CK(cp(o->del_qual, rc.del_qual + b, 4 * n));
  CK(cp(o->insertions, rc.insertions + b, 4 * n));
  CK(cp(o->ins_qual, rc.ins_qual + b, 4 * n));
  CK(cp(o->clips, rc.clips + b, 4 * n));
  CK(cp(o->call, rc.call + b, 4 * n));
  CK(cp(o->score, rc.score + b, 8 * n));
  CK(cp(o->indel_len, rc.indel_len + b, 4 * n));
  CK(cp(o->ins_str, rc.ins_str + b, 4 * n));
  unsigned long long pool_fill = 0;
  CK(cudaMemcpyAsync(&pool_fill, P<unsigned long long>(c->counters) + CNT_POOL, sizeof pool_fill,
                     cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (o->ins_chars) {
    if ((int64_t)pool_fill > o->ins_chars_cap)
      return fail(c, PG_ERR_LIMIT, "ins_chars needs %llu bytes", (unsigned long long)pool_fill);
    if (pool_fill) CK(cudaMemcpyAsync(o->ins_chars, c->pool.p, pool_fill, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  o->ins_chars_cap = (int64_t)pool_fill;
  return PG_OK;
}

pg_status pg_fetch_region(pg_ctx* c, int32_t r, pg_region_out* o) try {
  const Range nvtx_range("pg_fetch_region");
  if (!c || !o) return PG_ERR_ARG;
  if (!c->have_results) return fail(c, PG_ERR_STATE, "no results: run pg_pileup_regions first");
  if (r < 0 || r >= c->n_regions) return fail(c, PG_ERR_ARG, "region %d out of range", r);
  cudaSetDevice(c->device);
  const RegionDev& g = c->regions_h[r];
  return fetch_positions(c, g.pos_base, (size_t)g.size, o);
} PG_HOST_CATCH(c)

pg_status pg_fetch_all(pg_ctx* c, pg_region_out* o) try {
  const Range nvtx_range("pg_fetch_all");
  if (!c || !o) return PG_ERR_ARG;
  if (!c->have_results) return fail(c, PG_ERR_STATE, "no results: run pg_pileup_regions first");
  cudaSetDevice(c->device);
  return fetch_positions(c, 0, (size_t)c->n_positions, o);
} PG_HOST_CATCH(c)

pg_status pg_fetch_changes(pg_ctx* c, pg_change* out, int64_t cap, int64_t* n_changes, char* ins_chars,
                           int64_t ins_cap, int64_t* n_ins_chars) try {
  const Range nvtx_range("pg_fetch_changes");
  if (!c || !n_changes || !n_ins_chars || cap < 0 || (cap > 0 && !out) || ins_cap < 0)
    return fail(c, PG_ERR_ARG, "bad arguments");
  if (!c->have_results) return fail(c, PG_ERR_STATE, "no results: run pg_pileup_regions first");
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  *n_changes = *n_ins_chars = 0;
  const int32_t nt = c->n_call_tiles;
  if (nt == 0) return PG_OK;
  pg_status s;
  if ((s = ensure(c, c->chg_count, 4 * ((size_t)nt + 2)))) return s;
  if ((s = ensure(c, c->chg_off, 4 * ((size_t)nt + 2)))) return s;
  launch_change_count(P<RegionDev>(c->regions), P<int32_t>(c->call_tile_region), P<uint32_t>(c->rec_call),
                      P<int32_t>(c->chg_count), nt, st);
  launch_scan_small(P<int32_t>(c->chg_count), P<int32_t>(c->chg_off), nt, st);
  int32_t total = 0;
  unsigned long long pool_fill = 0;
  CK(cudaMemcpyAsync(&total, P<int32_t>(c->chg_off) + nt, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&pool_fill, P<unsigned long long>(c->counters) + CNT_POOL, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if ((s = ensure(c, c->chg_out, sizeof(pg_change) * (size_t)std::max(total, 1)))) return s;
  launch_change_write(P<RegionDev>(c->regions), P<int32_t>(c->call_tile_region), records(c),
                      P<int32_t>(c->chg_count), P<int32_t>(c->chg_off), P<pg_change>(c->chg_out), nt, st);
  CK(cudaGetLastError());
  const int64_t ncopy = std::min<int64_t>(total, cap);
  if (ncopy > 0) CK(cudaMemcpyAsync(out, c->chg_out.p, sizeof(pg_change) * ncopy, cudaMemcpyDeviceToHost, st));
  if (ins_chars && pool_fill > 0 && (int64_t)pool_fill <= ins_cap)
    CK(cudaMemcpyAsync(ins_chars, c->pool.p, pool_fill, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *n_changes = total;
  *n_ins_chars = (int64_t)pool_fill;
  return PG_OK;
} PG_HOST_CATCH(c)

static int64_t next_pow2(int64_t x) {
  int64_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

static pg_status kmer_core(pg_ctx* c, int32_t n_windows, int32_t K, const pg_params* params, int32_t min_depth,
                           bool wide, void* edges, int64_t cap, int64_t* n_edges, const int64_t* rlist = nullptr);
static pg_status kmer_windows(pg_ctx* c, const pg_window* windows, int32_t n_windows, int32_t K,
                              const pg_params* params, int32_t min_depth, bool wide, void* edges, int64_t cap,
                              int64_t* n_edges, int64_t n_list = 0, const int64_t* rlist = nullptr);

pg_status pg_kmer_tally(pg_ctx* c, const pg_window* windows, int32_t n_windows, int32_t K, const pg_params* params,
                        int32_t min_depth, pg_kmer_edge* edges, int64_t cap, int64_t* n_edges) try {
  const Range nvtx_range("pg_kmer_tally");
  if (c && (K < 1 || K > 31))
    return fail(c, PG_ERR_LIMIT, "K = %d: pg_kmer_tally packs K-mers in 64 bits (K <= 31); pg_kmer_tally_wide "
                "takes K <= 63", K);
  return kmer_windows(c, windows, n_windows, K, params, min_depth, false, edges, cap, n_edges);
} PG_HOST_CATCH(c)

pg_status pg_kmer_tally_wide(pg_ctx* c, const pg_window* windows, int32_t n_windows, int32_t K,
                             const pg_params* params, int32_t min_depth, pg_kmer_edge_wide* edges, int64_t cap,
                             int64_t* n_edges) try {
  const Range nvtx_range("pg_kmer_tally_wide");
  if (c && (K < 1 || K > 63)) return fail(c, PG_ERR_LIMIT, "K = %d: pg_kmer_tally_wide takes K <= 63", K);
  return kmer_windows(c, windows, n_windows, K, params, min_depth, true, edges, cap, n_edges);
} PG_HOST_CATCH(c)

pg_status pg_kmer_tally_reads(pg_ctx* c, const int64_t* reads, int64_t n_reads, const pg_window* windows,
                              int32_t n_windows, int32_t K, const pg_params* params, int32_t min_depth,
                              pg_kmer_edge_wide* edges, int64_t cap, int64_t* n_edges) try {
  const Range nvtx_range("pg_kmer_tally_reads");
  if (!c) return PG_ERR_ARG;
  if (K < 1 || K > 63) return fail(c, PG_ERR_LIMIT, "K = %d: pg_kmer_tally_reads takes K <= 63", K);
  if (n_reads < 0 || (n_reads > 0 && !reads) || (n_windows > 0 && !windows) || n_windows < 0)
    return fail(c, PG_ERR_ARG, "bad arguments");
  if (!c->have_reads) return fail(c, PG_ERR_STATE, "pg_set_reads must come first");
  for (int64_t k = 0; k < n_reads; k++)
    if (reads[k] < 0 || reads[k] >= c->R.n) return fail(c, PG_ERR_ARG, "read list entry %lld out of bounds", (long long)k);
  for (int32_t w = 0; w < n_windows; w++)
    if (windows[w].read_begin < 0 || windows[w].read_end < windows[w].read_begin || windows[w].read_end > n_reads)
      return fail(c, PG_ERR_ARG, "window %d: range outside the read list", w);
  cudaSetDevice(c->device);
  pg_status s;
  if ((s = ensure(c, c->klist, 8 * (size_t)std::max<int64_t>(n_reads, 1)))) return s;
  if (n_reads > 0) CK(cudaMemcpyAsync(c->klist.p, reads, 8 * (size_t)n_reads, cudaMemcpyHostToDevice, c->stream));
  return kmer_windows(c, windows, n_windows, K, params, min_depth, true, edges, cap, n_edges, n_reads,
                      P<int64_t>(c->klist));
} PG_HOST_CATCH(c)

static pg_status kmer_windows(pg_ctx* c, const pg_window* windows, int32_t n_windows, int32_t K,
                              const pg_params* params, int32_t min_depth, bool wide, void* edges, int64_t cap,
                              int64_t* n_edges, int64_t n_list, const int64_t* rlist) {
  if (!c || (n_windows > 0 && !windows) || !params || n_windows < 0 || cap < 0 || !n_edges)
    return fail(c, PG_ERR_ARG, "bad arguments");
  if (min_depth < 1) return fail(c, PG_ERR_ARG, "min_depth must be >= 1");
  if (params->min_qual < 0) return fail(c, PG_ERR_ARG, "min_qual must be >= 0");
  if (pg_status s0 = check_default_qual(c, params)) return s0;
  if (!c->have_reads) return fail(c, PG_ERR_STATE, "pg_set_reads must come first");
  cudaSetDevice(c->device);
  *n_edges = 0;
  if (n_windows == 0) return PG_OK;
  const int64_t n_idx = rlist ? n_list : c->R.n;
  for (int32_t w = 0; w < n_windows; w++)
    if (windows[w].read_begin < 0 || windows[w].read_end < windows[w].read_begin || windows[w].read_end > n_idx)
      return fail(c, PG_ERR_ARG, "window %d: read range out of bounds", w);
  pg_status s;
  if ((s = ensure(c, c->kwin, sizeof(pg_window) * n_windows))) return s;
  CK(cudaMemcpyAsync(c->kwin.p, windows, sizeof(pg_window) * n_windows, cudaMemcpyHostToDevice, c->stream));
  return kmer_core(c, n_windows, K, params, min_depth, wide, edges, cap, n_edges, rlist);
}

// The tally over the n_windows windows in c->kwin (device).
//
// Tables are sized at a quarter of each window's K-mer events (the distinct
// K-mers are fewer: every error-free K-mer recurs once per covering read and
// strand; 13% of the events on the 120 Mb workload) and windows are grouped
// into batches of about kTallyBatchBytes of tables, so that a batch's probes
// and counter atomics stay in L2.  A batch of a few dozen windows still fills
// the GPU: one warp per read, CTAs of kTallyReadsPerChunk reads.  The batches
// run back to back on the stream with no host wait; a window whose table fills
// up (a probe sequence longer than the kernel's bound) writes no edges and is
// counted again, after all batches, with a table four times larger.  The
// results do not depend on the table size or the batching.
constexpr int64_t kTallyBatchBytes = (int64_t)64 << 20;
constexpr int64_t kTallyReadsPerChunk = 8;

static pg_status kmer_core(pg_ctx* c, int32_t n_windows, int32_t K, const pg_params* params, int32_t min_depth,
                           bool wide, void* edges, int64_t cap, int64_t* n_edges, const int64_t* rlist) {
  cudaStream_t st = c->stream;
  // bytes per slot: KmerSlot / KmerSlotWide; exotic slots hold 2 or 4 key words, a used byte and
  // the counters (rounded up)
  const int64_t slot_b = wide ? (int64_t)sizeof(KmerSlotWide) : (int64_t)sizeof(KmerSlot);
  const int64_t xkw = wide ? 4 : 2;
  const size_t edge_b = wide ? sizeof(pg_kmer_edge_wide) : sizeof(pg_kmer_edge);
  pg_status s;
  c->tally_ms = 0;
  c->tally_events = c->tally_distinct = c->tally_max_batch_bytes = 0;
  c->tally_batches = 0;
  if ((s = ensure(c, c->kpre, sizeof(long long) * 3 * n_windows))) return s;
  launch_kmer_prepass(c->R, P<pg_window>(c->kwin), rlist, n_windows, K, P<long long>(c->kpre), st);
  std::vector<long long> pre(3 * (size_t)n_windows);
  std::vector<pg_window> wins(n_windows);
  CK(cudaMemcpyAsync(pre.data(), c->kpre.p, sizeof(long long) * pre.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(wins.data(), c->kwin.p, sizeof(pg_window) * wins.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::vector<int64_t> sbase(n_windows), scap(n_windows), xbase(n_windows), xcap(n_windows), evbase(n_windows),
      evcap(n_windows);
  for (int32_t w = 0; w < n_windows; w++) {
    // Assembler.addRead prunes K-mers with count < 2 every 100,000 reads
    // (S/Assembler.scala:74), which makes the tally order dependent.
    if (pre[3 * w] >= 100000)
      return fail(c, PG_ERR_LIMIT, "window %d has %lld reads; the tally is exact below 100,000", w, pre[3 * w]);
    scap[w] = next_pow2(std::max<int64_t>(256, pre[3 * w + 1] / 4));
    xcap[w] = pre[3 * w + 2] > 0 ? next_pow2(std::max<int64_t>(16, 2 * pre[3 * w + 2])) : 0;
    evcap[w] = pre[3 * w + 2];
    c->tally_events += pre[3 * w + 1];
  }
  const int64_t edge_cap = std::max<int64_t>(cap, 1);
  const size_t nwb = (size_t)std::max<int32_t>(n_windows, 1);
  if ((s = ensure(c, c->kedges, edge_b * edge_cap))) return s;
  if ((s = ensure(c, c->kcount, 16))) return s;
  if ((s = ensure(c, c->kwflag, 4 * nwb))) return s;
  if ((s = ensure(c, c->kused, 8 * nwb))) return s;
  if ((s = ensure(c, c->kwlist, 4 * nwb))) return s;
  if ((s = ensure(c, c->kslot_base, 8 * nwb))) return s;
  if ((s = ensure(c, c->kslot_cap, 8 * nwb))) return s;
  if ((s = ensure(c, c->kx_base, 8 * nwb))) return s;
  if ((s = ensure(c, c->kx_cap, 8 * nwb))) return s;
  if ((s = ensure(c, c->kx_evbase, 8 * nwb))) return s;
  if ((s = ensure(c, c->kx_evcap, 8 * nwb))) return s;
  if ((s = ensure(c, c->kx_evfill, 8 * nwb))) return s;
  CK(cudaMemsetAsync(c->kcount.p, 0, 16, st));
  CK(cudaMemsetAsync(c->kused.p, 0, 8 * nwb, st));
  CK(cudaMemsetAsync(c->kwflag.p, 0, 4 * nwb, st));
  CK(cudaMemsetAsync(c->kx_evfill.p, 0, 8 * nwb, st));
  auto table_bytes = [&](int32_t w) { return scap[w] * slot_b; };
  struct Batch {
    int32_t l0, l1;  // windows list[l0, l1)
    int64_t c0, c1;  // chunks [c0, c1)
    int64_t ns;      // table slots
  };
  std::vector<int32_t> list(n_windows);
  for (int32_t w = 0; w < n_windows; w++) list[w] = w;
  std::vector<KmerChunk> chunks;
  std::vector<Batch> batches;
  KmerArgs a;
  a.R = c->R; a.rlist = rlist; a.K = K; a.wide = wide;
  a.min_qual = params->min_qual; a.default_qual = params->default_qual; a.min_depth = min_depth;
  a.full = P<int32_t>(c->kwflag); a.used = P<unsigned long long>(c->kused);
  a.slot_base = P<int64_t>(c->kslot_base); a.slot_cap = P<int64_t>(c->kslot_cap);
  a.x_base = P<int64_t>(c->kx_base); a.x_cap = P<int64_t>(c->kx_cap);
  a.x_ev_base = P<int64_t>(c->kx_evbase); a.x_ev_cap = P<int64_t>(c->kx_evcap);
  a.x_ev_fill = P<unsigned long long>(c->kx_evfill);
  a.edges = P<pg_kmer_edge>(c->kedges); a.wedges = P<pg_kmer_edge_wide>(c->kedges); a.edge_cap = edge_cap;
  a.n_edges = P<unsigned long long>(c->kcount); a.overflow = (int32_t*)(P<unsigned long long>(c->kcount) + 1);
  for (int pass = 0; !list.empty(); pass++) {
    if (pass > 8) return fail(c, PG_ERR_LIMIT, "K-mer table overflow");
    // batches over the listed windows; table offsets are relative to the batch
    batches.clear();
    chunks.clear();
    int64_t max_ns = 1, nx = 0, ne = 0;
    for (int32_t w : list) {  // exotic tables and event lists: the whole pass
      xbase[w] = nx; evbase[w] = ne;
      nx += xcap[w]; ne += evcap[w];
    }
    nx = std::max<int64_t>(nx, 1);
    ne = std::max<int64_t>(ne, 1);
    for (int32_t l0 = 0; l0 < (int32_t)list.size();) {
      Batch b{l0, l0, (int64_t)chunks.size(), 0, 0};
      int64_t bytes = 0;
      while (b.l1 < (int32_t)list.size() && (b.l1 == l0 || bytes + table_bytes(list[b.l1]) <= kTallyBatchBytes)) {
        const int32_t w = list[b.l1++];
        bytes += table_bytes(w);
        sbase[w] = b.ns;
        b.ns += scap[w];
        for (int64_t lo = wins[w].read_begin; lo < wins[w].read_end; lo += kTallyReadsPerChunk)
          chunks.push_back(KmerChunk{lo, std::min<int64_t>(lo + kTallyReadsPerChunk, wins[w].read_end), w, 0});
      }
      b.c1 = (int64_t)chunks.size();
      max_ns = std::max(max_ns, b.ns);
      c->tally_max_batch_bytes = std::max(c->tally_max_batch_bytes, bytes);
      batches.push_back(b);
      l0 = b.l1;
    }
    if ((s = ensure(c, c->kslots, (size_t)(slot_b * max_ns)))) return s;
    if ((s = ensure(c, c->kx_ev, 16 * (size_t)ne))) return s;
    if ((s = ensure(c, c->kx_keys, 8 * xkw * (size_t)nx))) return s;
    if ((s = ensure(c, c->kx_used, (size_t)nx))) return s;
    if ((s = ensure(c, c->kx_cnt, 16 * (size_t)nx))) return s;
    if ((s = ensure(c, c->kx_qs, 32 * (size_t)nx))) return s;
    if ((s = ensure(c, c->kx_q, 4 * (size_t)nx))) return s;
    if ((s = ensure(c, c->kchunks, sizeof(KmerChunk) * std::max<size_t>(chunks.size(), 1)))) return s;
    if (!chunks.empty())
      CK(cudaMemcpyAsync(c->kchunks.p, chunks.data(), sizeof(KmerChunk) * chunks.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->kwlist.p, list.data(), 4 * list.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->kslot_base.p, sbase.data(), 8 * (size_t)n_windows, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->kslot_cap.p, scap.data(), 8 * (size_t)n_windows, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->kx_base.p, xbase.data(), 8 * (size_t)n_windows, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->kx_cap.p, xcap.data(), 8 * (size_t)n_windows, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->kx_evbase.p, evbase.data(), 8 * (size_t)n_windows, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->kx_evcap.p, evcap.data(), 8 * (size_t)n_windows, cudaMemcpyHostToDevice, st));
    a.slots = c->kslots.p;
    a.x_keys = P<unsigned long long>(c->kx_keys); a.x_used = P<uint8_t>(c->kx_used);
    a.x_cnt = P<uint32_t>(c->kx_cnt); a.x_qs = P<unsigned long long>(c->kx_qs); a.x_q = P<uint32_t>(c->kx_q);
    a.x_events = P<longlong2>(c->kx_ev);
    CK(cudaEventRecord(c->e0, st));
    if (pass > 0) {  // the windows counted again start from zero
      a.win_list = P<int32_t>(c->kwlist); a.n_win = (int32_t)list.size();
      launch_kmer_reset(a, st);
    }
    CK(cudaMemsetAsync(c->kx_used.p, 0, (size_t)nx, st));
    CK(cudaMemsetAsync(c->kx_cnt.p, 0, 16 * (size_t)nx, st));
    CK(cudaMemsetAsync(c->kx_qs.p, 0, 32 * (size_t)nx, st));
    CK(cudaMemsetAsync(c->kx_q.p, 0, 4 * (size_t)nx, st));
    for (const Batch& b : batches) {
      CK(cudaMemsetAsync(c->kslots.p, 0, (size_t)(slot_b * b.ns), st));
      a.win_list = P<int32_t>(c->kwlist) + b.l0; a.n_win = b.l1 - b.l0;
      a.chunks = P<KmerChunk>(c->kchunks) + b.c0; a.n_chunks = (int32_t)(b.c1 - b.c0);
      launch_kmer_count(a, st);
      launch_kmer_edges(a, st);
      c->tally_batches++;
    }
    // the exotic K-mers of every window of the pass, a warp per window (windows
    // found full skip theirs: they are counted again, exotic K-mers included)
    a.win_list = P<int32_t>(c->kwlist); a.n_win = (int32_t)list.size();
    launch_kmer_exotic(a, st);
    CK(cudaEventRecord(c->e1, st));
    CK(cudaGetLastError());
    std::vector<int32_t> all(n_windows);
    CK(cudaMemcpyAsync(all.data(), c->kwflag.p, 4 * (size_t)n_windows, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->e0, c->e1));
    c->tally_ms += ms;
    std::vector<int32_t> again;
    for (int32_t w : list)
      if (all[w]) {
        again.push_back(w);
        scap[w] *= 4;
      }
    list.swap(again);
  }
  unsigned long long hc[2];
  std::vector<unsigned long long> used(n_windows);
  CK(cudaMemcpyAsync(hc, c->kcount.p, 16, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(used.data(), c->kused.p, 8 * (size_t)n_windows, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (unsigned long long u : used) c->tally_distinct += (int64_t)u;
  if ((int32_t)hc[1]) return fail(c, PG_ERR_LIMIT, "K-mer table overflow");
  *n_edges = (int64_t)hc[0];
  const int64_t ncopy = std::min<int64_t>((int64_t)hc[0], cap);
  if (ncopy > 0 && edges) {
    CK(cudaMemcpyAsync(edges, c->kedges.p, edge_b * ncopy, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  return PG_OK;
}

// Finds the breaks of the last pileup call on the device (once per call and
// min_min_depth); they stay in c->bout, ordered by region and position.
static pg_status find_breaks_device(pg_ctx* c, int32_t min_min_depth) {
  if (c->brk_n >= 0 && c->brk_mmd == min_min_depth) return PG_OK;
  cudaStream_t st = c->stream;
  pg_status s;
  const size_t runs = (size_t)c->n_call_tiles * (kBreakStarts + 1);
  if ((s = ensure(c, c->bfrag, 4 * (size_t)std::max<int64_t>(c->n_positions, 1)))) return s;
  if ((s = ensure(c, c->bsums, 24 * (size_t)c->n_regions))) return s;
  if ((s = ensure(c, c->btiles, sizeof(BreakTile) * (size_t)c->n_call_tiles))) return s;
  if ((s = ensure(c, c->bgaps, sizeof(int2) * runs))) return s;
  if ((s = ensure(c, c->bruns, sizeof(int2) * runs))) return s;
  if ((s = ensure(c, c->bcnt, 4 * ((size_t)c->n_regions + 1)))) return s;
  if ((s = ensure(c, c->boff, 4 * ((size_t)c->n_regions + 1)))) return s;
  if ((s = ensure(c, c->bout, sizeof(pg_break) * runs))) return s;
  CK(cudaMemsetAsync(c->bsums.p, 0, 24 * (size_t)c->n_regions, st));
  CK(cudaMemsetAsync(c->bcnt.p, 0, 4 * ((size_t)c->n_regions + 1), st));
  BreakArgs a;
  a.regions = P<RegionDev>(c->regions); a.call_tile_region = P<int32_t>(c->call_tile_region);
  a.tile_begin = 0; a.n_tiles = c->n_call_tiles; a.rec = records(c); a.stats = P<StatsDev>(c->stats);
  a.ref = P<uint8_t>(c->ref); a.min_min_depth = min_min_depth; a.frag = P<int32_t>(c->bfrag);
  a.sums = P<long long>(c->bsums); a.tiles = P<BreakTile>(c->btiles); a.gap_scratch = P<int2>(c->bgaps);
  a.brk_scratch = P<int2>(c->bruns); a.brk_count = P<int32_t>(c->bcnt); a.brk_off = P<int32_t>(c->boff);
  a.out = P<pg_break>(c->bout);
  launch_breaks(a, c->n_regions, st);
  CK(cudaGetLastError());
  int32_t n = 0;
  CK(cudaMemcpyAsync(&n, P<int32_t>(c->boff) + c->n_regions, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  c->brk_n = n;
  c->brk_mmd = min_min_depth;
  return PG_OK;
}

pg_status pg_find_breaks(pg_ctx* c, int32_t min_min_depth, pg_break* out, int64_t cap, int64_t* n_breaks) try {
  const Range nvtx_range("pg_find_breaks");
  if (!c || !n_breaks || cap < 0 || (cap > 0 && !out)) return fail(c, PG_ERR_ARG, "bad arguments");
  if (!c->have_results) return fail(c, PG_ERR_STATE, "no pileup results: call pg_pileup_regions first");
  cudaSetDevice(c->device);
  *n_breaks = 0;
  if (c->n_regions == 0 || c->n_call_tiles == 0) return PG_OK;
  pg_status s = find_breaks_device(c, min_min_depth);
  if (s) return s;
  *n_breaks = c->brk_n;
  const int64_t ncopy = std::min<int64_t>(c->brk_n, cap);
  if (ncopy > 0) {
    CK(cudaMemcpyAsync(out, c->bout.p, sizeof(pg_break) * (size_t)ncopy, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return PG_OK;
} PG_HOST_CATCH(c)

pg_status pg_find_duplications(pg_ctx* c, pg_break* out, int64_t cap, int64_t* n_dups) try {
  const Range nvtx_range("pg_find_duplications");
  if (!c || !n_dups || cap < 0 || (cap > 0 && !out)) return fail(c, PG_ERR_ARG, "bad arguments");
  if (!c->have_results) return fail(c, PG_ERR_STATE, "no pileup results: call pg_pileup_regions first");
  cudaSetDevice(c->device);
  *n_dups = 0;
  if (c->n_regions == 0 || c->n_call_tiles == 0) return PG_OK;
  // fragCoverage and its region sums are made with the break candidates
  pg_status s = find_breaks_device(c, c->brk_n >= 0 ? c->brk_mmd : 5);
  if (s) return s;
  cudaStream_t st = c->stream;
  const int64_t dcap = c->n_positions / 2000 + c->n_regions + 16;  // runs are > 2001 apart
  if ((s = ensure(c, c->druns, sizeof(int2) * (size_t)c->n_call_tiles))) return s;
  if ((s = ensure(c, c->dout, sizeof(pg_break) * (size_t)dcap))) return s;
  if ((s = ensure(c, c->dcount, 8))) return s;
  CK(cudaMemsetAsync(c->dcount.p, 0, 8, st));
  BreakArgs a;
  a.regions = P<RegionDev>(c->regions); a.call_tile_region = P<int32_t>(c->call_tile_region);
  a.tile_begin = 0; a.n_tiles = c->n_call_tiles; a.rec = records(c); a.stats = P<StatsDev>(c->stats);
  a.ref = P<uint8_t>(c->ref); a.min_min_depth = c->brk_mmd; a.frag = P<int32_t>(c->bfrag);
  a.sums = P<long long>(c->bsums);
  launch_duplications(a, c->n_regions, P<int2>(c->druns), P<pg_break>(c->dout), dcap,
                      P<unsigned long long>(c->dcount), st);
  CK(cudaGetLastError());
  unsigned long long n = 0;
  CK(cudaMemcpyAsync(&n, c->dcount.p, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::vector<pg_break> v(std::min<uint64_t>(n, (uint64_t)dcap));
  if (!v.empty())
    CK(cudaMemcpyAsync(v.data(), c->dout.p, sizeof(pg_break) * v.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::sort(v.begin(), v.end(), [](const pg_break& x, const pg_break& y) {
    return x.region != y.region ? x.region < y.region : x.start < y.start;
  });
  *n_dups = (int64_t)v.size();
  for (int64_t k = 0; k < std::min<int64_t>(cap, (int64_t)v.size()); k++) out[k] = v[k];
  return PG_OK;
} PG_HOST_CATCH(c)

static pg_status kmer_breaks(pg_ctx* c, int32_t min_min_depth, int32_t radius, int32_t K, const pg_params* params,
                             int32_t min_depth, bool wide, void* edges, int64_t cap, int64_t* n_windows,
                             int64_t* n_edges);

pg_status pg_kmer_tally_breaks(pg_ctx* c, int32_t min_min_depth, int32_t radius, int32_t K, const pg_params* params,
                               int32_t min_depth, pg_kmer_edge* edges, int64_t cap, int64_t* n_windows,
                               int64_t* n_edges) try {
  const Range nvtx_range("pg_kmer_tally_breaks");
  if (c && (K < 1 || K > 31))
    return fail(c, PG_ERR_LIMIT, "K = %d: pg_kmer_tally_breaks packs K-mers in 64 bits (K <= 31); "
                "pg_kmer_tally_breaks_wide takes K <= 63", K);
  return kmer_breaks(c, min_min_depth, radius, K, params, min_depth, false, edges, cap, n_windows, n_edges);
} PG_HOST_CATCH(c)

pg_status pg_kmer_tally_breaks_wide(pg_ctx* c, int32_t min_min_depth, int32_t radius, int32_t K,
                                    const pg_params* params, int32_t min_depth, pg_kmer_edge_wide* edges,
                                    int64_t cap, int64_t* n_windows, int64_t* n_edges) try {
  const Range nvtx_range("pg_kmer_tally_breaks_wide");
  if (c && (K < 1 || K > 63)) return fail(c, PG_ERR_LIMIT, "K = %d: pg_kmer_tally_breaks_wide takes K <= 63", K);
  return kmer_breaks(c, min_min_depth, radius, K, params, min_depth, true, edges, cap, n_windows, n_edges);
} PG_HOST_CATCH(c)

static pg_status kmer_breaks(pg_ctx* c, int32_t min_min_depth, int32_t radius, int32_t K, const pg_params* params,
                             int32_t min_depth, bool wide, void* edges, int64_t cap, int64_t* n_windows,
                             int64_t* n_edges) {
  if (!c || !params || cap < 0 || !n_edges || !n_windows || radius < 0) return fail(c, PG_ERR_ARG, "bad arguments");
  if (min_depth < 1) return fail(c, PG_ERR_ARG, "min_depth must be >= 1");
  if (params->min_qual < 0) return fail(c, PG_ERR_ARG, "min_qual must be >= 0");
  if (pg_status s0 = check_default_qual(c, params)) return s0;
  if (!c->have_results) return fail(c, PG_ERR_STATE, "no pileup results: call pg_pileup_regions first");
  cudaSetDevice(c->device);
  *n_edges = 0;
  *n_windows = 0;
  if (c->n_regions == 0 || c->n_call_tiles == 0) return PG_OK;
  pg_status s = find_breaks_device(c, min_min_depth);
  if (s) return s;
  const int32_t n = (int32_t)c->brk_n;
  *n_windows = n;
  if (n == 0) return PG_OK;
  if ((s = ensure(c, c->kwin, sizeof(pg_window) * (size_t)n))) return s;
  launch_break_windows(c->R, P<RegionDev>(c->regions), P<pg_break>(c->bout), n, radius, P<ReadExtent>(c->d_ext),
                       P<pg_window>(c->kwin), c->stream);
  CK(cudaGetLastError());
  return kmer_core(c, n, K, params, min_depth, wide, edges, cap, n_edges);
}

pg_status pg_mark_deleted(pg_ctx* c, int32_t r, int32_t first_locus, int32_t count) try {
  if (!c || count < 0) return fail(c, PG_ERR_ARG, "bad arguments");
  if (!c->have_results) return fail(c, PG_ERR_STATE, "no results: run pg_pileup_regions first");
  if (r < 0 || r >= c->n_regions) return fail(c, PG_ERR_ARG, "region %d out of range", r);
  const RegionDev& g = c->regions_h[r];
  if (count == 0) return PG_OK;
  if (first_locus < g.start || (int64_t)first_locus + count - 1 > (int64_t)g.stop)
    return fail(c, PG_ERR_ARG, "loci %d..%lld outside region %d", first_locus, (long long)first_locus + count - 1, r);
  cudaSetDevice(c->device);
  launch_mark_deleted(P<uint32_t>(c->rec_call) + g.pos_base + (first_locus - g.start), count, c->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return PG_OK;
} PG_HOST_CATCH(c)

pg_status pg_format_vcf(pg_ctx* c, int32_t r, const char* name, int32_t diploid, int32_t vcf_qe,
                        int32_t variants_only, char* out, int64_t cap, int64_t* n_bytes) try {
  const Range nvtx_range("pg_format_vcf");
  if (!c || !name || !n_bytes || cap < 0) return fail(c, PG_ERR_ARG, "bad arguments");
  if (!c->have_results) return fail(c, PG_ERR_STATE, "no results: run pg_pileup_regions first");
  if (r < 0 || r >= c->n_regions) return fail(c, PG_ERR_ARG, "region %d out of range", r);
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  const RegionDev& g = c->regions_h[r];
  const int64_t n = g.size;
  const size_t nl = strlen(name);
  pg_status s;
  if ((s = ensure(c, c->vlen, 8 * (size_t)n))) return s;
  if ((s = ensure(c, c->vsums, 8 * (size_t)((n + 1023) / 1024 + 2)))) return s;
  if ((s = ensure(c, c->vname, nl + 1))) return s;
  CK(cudaMemcpyAsync(c->vname.p, name, nl + 1, cudaMemcpyHostToDevice, st));
  FormatArgs A;
  A.region = g;
  A.rec = records(c);
  A.ref = P<uint8_t>(c->ref);
  A.pool = P<char>(c->pool);
  A.name = P<char>(c->vname);
  A.name_len = (int32_t)nl;
  A.min_depth = c->stats_h[r].min_depth;
  A.diploid = diploid;
  A.vcf_qe = vcf_qe;
  A.variants_only = variants_only;
  launch_vcf_lengths(A, P<int64_t>(c->vlen), st);
  launch_scan64(P<int64_t>(c->vlen), n, P<int64_t>(c->vsums), st);
  int64_t total = 0;
  const int32_t nb = (int32_t)((n + 1023) / 1024);
  CK(cudaMemcpyAsync(&total, P<int64_t>(c->vsums) + nb, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *n_bytes = total;
  if (total > cap) return fail(c, PG_ERR_LIMIT, "VCF text needs %lld bytes", (long long)total);
  if ((s = ensure(c, c->vtext, (size_t)std::max<int64_t>(total, 1)))) return s;
  launch_vcf_write(A, P<int64_t>(c->vlen), P<char>(c->vtext), st);
  CK(cudaGetLastError());
  if (total && out) CK(cudaMemcpyAsync(out, c->vtext.p, (size_t)total, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return PG_OK;
} PG_HOST_CATCH(c)

pg_status pg_last_tally_stats(pg_ctx* c, double* kernel_ms, int64_t* kmer_events, int64_t* distinct_kmers,
                              int64_t* max_batch_table_bytes, int32_t* batches) try {
  if (!c) return PG_ERR_ARG;
  if (kernel_ms) *kernel_ms = c->tally_ms;
  if (kmer_events) *kmer_events = c->tally_events;
  if (distinct_kmers) *distinct_kmers = c->tally_distinct;
  if (max_batch_table_bytes) *max_batch_table_bytes = c->tally_max_batch_bytes;
  if (batches) *batches = c->tally_batches;
  return PG_OK;
} PG_HOST_CATCH(c)

pg_status pg_graph_replays(pg_ctx* c, int32_t* replays) try {
  if (!c || !replays) return PG_ERR_ARG;
  *replays = c->graph_replays;
  return PG_OK;
} PG_HOST_CATCH(c)

pg_status pg_last_kernel_ms(pg_ctx* c, double* walk_ms, double* total_ms, int32_t* launches) try {
  if (!c) return PG_ERR_ARG;
  if (walk_ms) *walk_ms = c->walk_ms;
  if (total_ms) *total_ms = c->total_ms;
  if (launches) *launches = c->launches;
  return PG_OK;
} PG_HOST_CATCH(c)

}  // extern "C"
