// pg_serve.cu — serving region-polish requests through the C ABI.
//
// A request is the work of `pilon --targets contig:start-stop --fix
// snps,indels --vcf --changes` on one region (S/GenomeFile.scala:215-250): the
// region's pileups and calls (pg_pileup_regions), its fix lists and fixed bases
// (GenomeRegion.identifyAndFixIssues / fixIssues, S/GenomeRegion.scala:307-414,
// 557-621), its changes lines (writeChanges, :645-657) and its VCF records
// (Vcf.writeRecord, S/Vcf.scala:74-176) whose ALT is not ".".
//
// The server uploads the reference and the read store once and keeps them
// resident.  Each of n_workers host threads owns an engine context (its own
// CUDA stream and buffers) that uses the resident store in place.  A free
// worker takes, from the head of the queue, every request whose device bytes
// still fit the budget beside the batches already running, and runs them as
// one batched call; requests that arrive meanwhile wait only until memory and
// a worker free up, and the batches of different workers overlap on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pilon_gb300.h"
#include "pg_host_guard.h"

namespace {

using Clock = std::chrono::steady_clock;

// Device bytes a request needs while its batch runs (the buffers
// pg_pileup_regions sizes per call): per position the 88-byte pileup record,
// the call record (flags, score, indel length, insertion offset: 20 B), the
// event index (4 B) and the candidate slots (1.5 B), rounded up to 116 B; per
// read fed to the region its read-chunk state and indel-list slot, 16 B.
constexpr int64_t kBytesPerPosition = 116;
constexpr int64_t kBytesPerRead = 16;
constexpr int64_t kSlop = 10000;  // BamFile.process queries the region +- 10 kb (S/BamFile.scala:117-119)

struct Job {
  pg_request req{};
  int64_t rb = 0, re = 0, bytes = 0;
  Clock::time_point submitted, started, finished;
  bool done = false;
  int32_t status = PG_OK;
  int32_t batch = 0;
  std::string fasta, changes, vcf, message;
};

struct Fix {
  int32_t locus;
  std::string was, patch;
};

}  // namespace

struct pg_server {
  int device = 0;
  pg_serve_config cfg{};
  pg_params params{};
  std::vector<std::string> names;
  std::vector<std::vector<uint8_t>> ref;
  std::vector<int64_t> lens;
  // read index of the coordinate-sorted store: each contig's reads and their positions
  std::vector<int32_t> pos;
  std::vector<int64_t> contig_lo, contig_hi;
  int64_t max_span = 0;
  // the resident read store
  void* dbuf[15] = {nullptr};
  pg_reads dreads{};
  std::vector<pg_ctx*> workers;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> queue;
  std::map<uint64_t, Job> jobs;
  uint64_t next_ticket = 1;
  int64_t in_flight = 0, peak_in_flight = 0, batches = 0;
  bool closing = false;
  std::string err;
};

namespace {

pg_status serr(pg_server* s, pg_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (s) s->err = buf;
  return st;
}

// Region.regionString (S/Region.scala:45)
std::string region_string(const std::string& name, int64_t s, int64_t e) {
  std::string r = name + ":" + std::to_string(s);
  if (e + 1 - s >= 2) r += "-" + std::to_string(e);
  return r;
}

// the polished contig name (S/GenomeFile.scala:137-140)
std::string new_name(const std::string& name) {
  const char* sep = name.find('|') == std::string::npos ? "_" : (name.back() == '|' ? "" : "|");
  return name + sep + "pilon";
}

// GenomeRegion.fixFixList (S/GenomeRegion.scala:557-593): stable sort by locus,
// then of two overlapping fixes keep the one with more bases (ties: the first).
std::vector<Fix> fix_fix_list(std::vector<Fix> fx) {
  std::stable_sort(fx.begin(), fx.end(), [](const Fix& a, const Fix& b) { return a.locus < b.locus; });
  std::vector<Fix> out;
  size_t k = 0;
  while (k < fx.size()) {
    if (k + 1 < fx.size()) {
      const Fix &f1 = fx[k], &f2 = fx[k + 1];
      const int64_t e1 = f1.locus + std::max<int64_t>((int64_t)f1.was.size() - 1, 0);
      const int64_t e2 = f2.locus + std::max<int64_t>((int64_t)f2.was.size() - 1, 0);
      if (f2.locus <= e1 && e2 >= f1.locus) {
        if (f1.was.size() + f1.patch.size() >= f2.was.size() + f2.patch.size()) fx[k + 1] = f1;
      } else {
        out.push_back(f1);
      }
    } else {
      out.push_back(fx[k]);
    }
    k++;
  }
  return out;
}

// GenomeRegion.fixIssues (S/GenomeRegion.scala:595-621)
void fix_issues(std::string& bases, int32_t start, const std::vector<Fix>& fixes) {
  const std::vector<Fix> fx = fix_fix_list(fixes);
  for (auto it = fx.rbegin(); it != fx.rend(); ++it) {
    const size_t s = (size_t)(it->locus - start);
    if (it->was.size() == it->patch.size()) bases.replace(s, it->patch.size(), it->patch);
    else bases.replace(s, it->was.size(), it->patch);
  }
}

// Bases.toIUPAC of two bases (S/Bases.scala:85-88)
char to_iupac(char a, char b) {
  static const char* kIupac = ".ACMGRSVTWYHKDBN";
  auto bit = [](char c) { return c == 'A' ? 1 : c == 'C' ? 2 : c == 'G' ? 4 : 8; };
  return kIupac[bit(a) | bit(b)];
}

// One request's answer from region r of the worker's last pileup call.
pg_status answer(pg_server* S, pg_ctx* ctx, int32_t r, Job& j) {
  const pg_request& q = j.req;
  const int32_t size = q.stop - q.start + 1;
  std::vector<uint32_t> call(size);
  std::vector<int32_t> ilen(size), istr(size);
  pg_region_out o{};
  o.call = call.data();
  o.indel_len = ilen.data();
  o.ins_str = istr.data();
  pg_status st = pg_fetch_region(ctx, r, &o);
  if (st) return st;
  std::vector<char> chars;
  if (o.ins_chars_cap > 0) {
    chars.resize((size_t)o.ins_chars_cap);
    pg_region_out o2{};
    o2.ins_chars = chars.data();
    o2.ins_chars_cap = (int64_t)chars.size();
    if ((st = pg_fetch_region(ctx, r, &o2))) return st;
  }
  const std::vector<uint8_t>& ref = S->ref[q.contig];
  const std::string& name = S->names[q.contig];
  // identifyAndFixIssues for snps, indels (and amb through the params):
  // the reference prepends, so each list is in descending locus order
  std::vector<Fix> snp, small;
  for (int32_t i = size - 1; i >= 0; i--) {
    const uint32_t f = call[i];
    const uint32_t kind = PG_CALL_CHANGE(f);
    if (!kind) continue;
    const int32_t loc = q.start + i;
    const char rb = (char)toupper(ref[loc - 1]);
    const char cb = (f & PG_CALL_HAS_BASE) ? "ACGT"[f & 3u] : 'N';
    const char alt = "ACGT"[(f >> 2) & 3u];
    if (kind == PG_CHANGE_SNP) {
      if (S->cfg.fix_snps) snp.push_back({loc, std::string(1, rb), std::string(1, cb)});
    } else if (kind == PG_CHANGE_AMB) {
      if (S->cfg.fix_snps) {
        if (S->cfg.iupac) small.push_back({loc, std::string(1, rb), std::string(1, to_iupac(cb, alt))});
        else snp.push_back({loc, std::string(1, rb), std::string(1, cb)});
      }
    } else if (kind == PG_CHANGE_INS) {
      if (S->cfg.fix_indels && istr[i] >= 0 && (size_t)istr[i] + (size_t)ilen[i] <= chars.size())
        small.push_back({loc, "", std::string(chars.data() + istr[i], (size_t)ilen[i])});
    } else if (kind == PG_CHANGE_DEL) {
      if (S->cfg.fix_indels) small.push_back({loc, std::string((const char*)ref.data() + loc - 1, (size_t)ilen[i]), ""});
    }
  }
  std::string bases((const char*)ref.data() + q.start - 1, (size_t)size);
  fix_issues(bases, q.start, snp);
  fix_issues(bases, q.start, small);
  j.fasta = std::move(bases);
  // writeChanges: each target is its own output entry, so the offset is 0
  std::vector<Fix> all = snp;
  all.insert(all.end(), small.begin(), small.end());
  const std::string nn = new_name(name);
  int64_t delta = 0;
  j.changes.clear();
  for (const Fix& f : fix_fix_list(all)) {
    const int64_t nl = f.locus + delta;
    j.changes += region_string(name, f.locus, f.locus + (int64_t)f.was.size() - 1) + " " +
                 region_string(nn, nl, nl + (int64_t)f.patch.size() - 1) + " " + (f.was.empty() ? "." : f.was) +
                 " " + (f.patch.empty() ? "." : f.patch) + "\n";
    delta += (int64_t)f.patch.size() - (int64_t)f.was.size();
  }
  // the region's VCF records whose ALT is not "." (device formatter)
  int64_t n = 0;
  st = pg_format_vcf(ctx, r, name.c_str(), S->cfg.diploid, S->cfg.vcf_qe, 1, nullptr, 0, &n);
  if (st && st != PG_ERR_LIMIT) return st;
  j.vcf.assign((size_t)n, '\0');
  if (n > 0 && (st = pg_format_vcf(ctx, r, name.c_str(), S->cfg.diploid, S->cfg.vcf_qe, 1, &j.vcf[0], n, &n)))
    return st;
  return PG_OK;
}

// A free worker's next batch: from the head of the queue, every request whose
// device bytes still fit the budget beside the batches in flight.  The batch's
// room is reserved before anything leaves the queue, so an allocation that
// fails here leaves the queue as it was.
void take(pg_server* S, std::unique_lock<std::mutex>& lk, int64_t& bytes, std::vector<Job*>& js) {
  js.clear();
  bytes = 0;
  for (;;) {
    if (S->closing && S->queue.empty()) return;
    if (!S->queue.empty() && S->in_flight + S->jobs[S->queue.front()].bytes <= S->cfg.hbm_budget) break;
    S->cv_work.wait(lk);
  }
  size_t count = 0;
  for (uint64_t t : S->queue) {
    const int64_t b = S->jobs[t].bytes;
    if (S->in_flight + bytes + b > S->cfg.hbm_budget) break;
    if (S->cfg.max_batch > 0 && (int32_t)count >= S->cfg.max_batch) break;
    bytes += b;
    count++;
  }
  js.reserve(count);
  for (size_t k = 0; k < count; k++) {
    js.push_back(&S->jobs[S->queue.front()]);  // map nodes stay put until released
    S->queue.pop_front();
  }
  S->in_flight += bytes;
  S->peak_in_flight = std::max(S->peak_in_flight, S->in_flight);
}

// A request that fails on a host exception: its status and message.
void fail_on_exception(Job& j) noexcept { j.status = pg::host_exception_status(&j.message); }

void worker(pg_server* S, pg_ctx* ctx) {
  cudaSetDevice(S->device);
  std::vector<pg_region> regions;
  std::vector<Job*> js;
  for (;;) {
    int64_t bytes = 0;
    int32_t bno = 0;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      try {
        take(S, lk, bytes, js);
      } catch (...) {
        // no room for a batch: the request at the head fails alone, so the queue still moves
        if (S->queue.empty()) continue;
        Job& j = S->jobs[S->queue.front()];
        S->queue.pop_front();
        fail_on_exception(j);
        j.finished = Clock::now();
        j.done = true;
        lk.unlock();
        S->cv_done.notify_all();
        continue;
      }
      if (js.empty()) return;
      bno = (int32_t)++S->batches;
    }
    const Clock::time_point t0 = Clock::now();
    for (Job* j : js) {
      j->started = t0;
      j->batch = bno;
    }
    pg_status st = PG_OK;
    std::string msg;
    try {
      regions.clear();
      regions.reserve(js.size());
      for (Job* j : js) regions.push_back(pg_region{j->req.contig, j->req.start, j->req.stop, 0, j->rb, j->re});
      st = pg_pileup_regions(ctx, regions.data(), (int32_t)regions.size(), &S->params, S->cfg.batched);
      if (st) msg = pg_last_error(ctx);
    } catch (...) {
      st = pg::host_exception_status(&msg);
    }
    for (size_t r = 0; r < js.size(); r++) {
      Job& j = *js[r];
      try {
        if (st == PG_OK || st == PG_ERR_INDEX) {
          pg_region_stats rs{};
          pg_status s2 = pg_fetch_stats(ctx, (int32_t)r, &rs);
          if (s2) { j.status = s2; j.message = pg_last_error(ctx); }
          else if (rs.error) {
            j.status = PG_ERR_INDEX;
            j.message = "an indel left shift leaves the target (Pilon throws ArrayIndexOutOfBoundsException)";
          } else if ((s2 = answer(S, ctx, (int32_t)r, j))) {
            j.status = s2;
            j.message = pg_last_error(ctx);
          }
        } else {
          j.status = st;
          j.message = msg;
        }
      } catch (...) {
        fail_on_exception(j);
      }
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      const Clock::time_point t1 = Clock::now();
      for (Job* j : js) {
        j->finished = t1;
        j->done = true;
      }
      S->in_flight -= bytes;
    }
    S->cv_work.notify_all();
    S->cv_done.notify_all();
  }
}

void free_store(pg_server* S) {
  for (void*& p : S->dbuf)
    if (p) {
      cudaFree(p);
      p = nullptr;
    }
}

}  // namespace

extern "C" {

void pg_default_serve_config(pg_serve_config* c) {
  if (!c) return;
  memset(c, 0, sizeof *c);
  c->device = 0;
  c->n_workers = 2;
  c->hbm_budget = (int64_t)8 << 30;
  c->fix_snps = 1;
  c->fix_indels = 1;
  c->batched = 1;
}

pg_status pg_serve_open(pg_server** out, const pg_serve_config* cfg, const pg_params* params, int32_t n_contigs,
                        const char* const* names, const int64_t* lens, const uint8_t* const* bases,
                        const pg_reads* h) try {
  if (!out) return PG_ERR_ARG;
  *out = nullptr;
  pg_server* S = new pg_server();
  *out = S;
  if (!cfg || !params || n_contigs < 0 || (n_contigs > 0 && (!names || !lens || !bases)) || !h || h->n_reads < 0)
    return serr(S, PG_ERR_ARG, "bad arguments");
  if (cfg->n_workers < 1 || cfg->n_workers > 64) return serr(S, PG_ERR_ARG, "n_workers must be in [1, 64]");
  if (cfg->hbm_budget <= 0) return serr(S, PG_ERR_ARG, "hbm_budget must be > 0");
  S->cfg = *cfg;
  S->params = *params;
  S->device = cfg->device;
  for (int32_t c = 0; c < n_contigs; c++) {
    if (!names[c] || lens[c] < 0 || (lens[c] > 0 && !bases[c])) return serr(S, PG_ERR_ARG, "contig %d", c);
    S->names.emplace_back(names[c]);
    S->lens.push_back(lens[c]);
    S->ref.emplace_back(bases[c], bases[c] + lens[c]);
  }
  // the read index: references in one run each, unplaced reads (negative) last
  const int64_t n = h->n_reads;
  int64_t placed = 0;
  for (int64_t i = 0; i < n; i++) {
    const int32_t rid = h->ref_id[i];
    if (rid >= 0) {
      if (placed != i || rid >= n_contigs || (i > 0 && rid < h->ref_id[i - 1]))
        return serr(S, PG_ERR_ARG, "reads are not coordinate-sorted (read %lld)", (long long)i);
      placed = i + 1;
    }
  }
  S->pos.assign(h->pos, h->pos + placed);
  S->contig_lo.assign(n_contigs, 0);
  S->contig_hi.assign(n_contigs, 0);
  int64_t k = 0;
  for (int32_t c = 0; c < n_contigs; c++) {
    while (k < placed && h->ref_id[k] < c) k++;
    S->contig_lo[c] = k;
    while (k < placed && h->ref_id[k] == c) k++;
    S->contig_hi[c] = k;
  }
  for (int64_t i = 0; i < placed; i++)
    S->max_span = std::max<int64_t>(S->max_span, (int64_t)h->aend[i] - h->pos[i] + 1);
  // the resident store, uploaded once
  if (cudaSetDevice(S->device) != cudaSuccess) {
    cudaGetLastError();
    return serr(S, PG_ERR_CUDA, "no CUDA device %d", S->device);
  }
  const void* src[15] = {h->pos, h->aend, h->tlen, h->ref_id, h->mate_ref_id, h->l_seq, h->flag, h->n_cigar,
                         h->mapq, h->seq, h->qual, h->cigar_off, h->seq_off, h->qual_off, h->cigar};
  const size_t nb[15] = {(size_t)n * 4, (size_t)n * 4, (size_t)n * 4, (size_t)n * 4, (size_t)n * 4, (size_t)n * 4,
                         (size_t)n * 2, (size_t)n * 2, (size_t)n, (size_t)h->seq_bytes, (size_t)h->qual_bytes,
                         (size_t)n * 8, (size_t)n * 8, (size_t)n * 8, (size_t)h->n_cigar_words * 4};
  for (int k = 0; k < 15; k++) {
    if (nb[k] && !src[k]) return serr(S, PG_ERR_ARG, "reads field %d is null", k);
    if (cudaMalloc(&S->dbuf[k], std::max<size_t>(nb[k], 16)) != cudaSuccess) {
      cudaGetLastError();
      free_store(S);
      return serr(S, PG_ERR_NOMEM, "device memory for the read store (%zu bytes)", nb[k]);
    }
    if (nb[k] && cudaMemcpy(S->dbuf[k], src[k], nb[k], cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      free_store(S);
      return serr(S, PG_ERR_CUDA, "upload of the read store failed");
    }
  }
  pg_reads& d = S->dreads;
  d = *h;
  d.pos = (const int32_t*)S->dbuf[0]; d.aend = (const int32_t*)S->dbuf[1]; d.tlen = (const int32_t*)S->dbuf[2];
  d.ref_id = (const int32_t*)S->dbuf[3]; d.mate_ref_id = (const int32_t*)S->dbuf[4];
  d.l_seq = (const int32_t*)S->dbuf[5]; d.flag = (const uint16_t*)S->dbuf[6];
  d.n_cigar = (const uint16_t*)S->dbuf[7]; d.mapq = (const uint8_t*)S->dbuf[8]; d.seq = (const uint8_t*)S->dbuf[9];
  d.qual = (const uint8_t*)S->dbuf[10]; d.cigar_off = (const int64_t*)S->dbuf[11];
  d.seq_off = (const int64_t*)S->dbuf[12]; d.qual_off = (const int64_t*)S->dbuf[13];
  d.cigar = (const uint32_t*)S->dbuf[14];
  std::vector<const uint8_t*> bp(n_contigs);
  for (int32_t c = 0; c < n_contigs; c++) bp[c] = S->ref[c].data();
  for (int32_t w = 0; w < cfg->n_workers; w++) {
    pg_ctx* ctx = nullptr;
    pg_status st = pg_open(&ctx, S->device);
    if (!st) st = pg_set_reference(ctx, n_contigs, S->lens.data(), bp.data());
    if (!st) st = pg_set_reads_device(ctx, &S->dreads);
    if (st) {
      S->err = ctx ? pg_last_error(ctx) : "pg_open failed";
      if (ctx) pg_close(ctx);
      for (pg_ctx* c2 : S->workers) pg_close(c2);
      S->workers.clear();
      free_store(S);
      return st;
    }
    S->workers.push_back(ctx);
  }
  for (pg_ctx* ctx : S->workers) S->threads.emplace_back(worker, S, ctx);
  return PG_OK;
} PG_HOST_CATCH(out ? *out : nullptr)

pg_status pg_serve_submit(pg_server* S, const pg_request* q, uint64_t* ticket) try {
  if (!S || !q || !ticket) return PG_ERR_ARG;
  if (S->threads.empty()) return serr(S, PG_ERR_STATE, "the server is not open");
  if (q->contig < 0 || q->contig >= (int32_t)S->lens.size() || q->start < 1 || q->stop < q->start ||
      q->stop > S->lens[q->contig])
    return serr(S, PG_ERR_ARG, "target %d:%d-%d outside the reference", q->contig, q->start, q->stop);
  Job j;
  j.req = *q;
  // the reads of the target's query window, as ReadIndex.range_for
  const int64_t lo = S->contig_lo[q->contig], hi = S->contig_hi[q->contig];
  const int64_t qs = std::max<int64_t>((int64_t)q->start - kSlop, 0);
  const int64_t qe = std::min<int64_t>((int64_t)q->stop + kSlop, S->lens[q->contig]);
  const int32_t* p0 = S->pos.data();
  j.rb = std::lower_bound(p0 + lo, p0 + hi, qs - S->max_span, [](int32_t a, int64_t v) { return a < v; }) - p0;
  j.re = std::upper_bound(p0 + lo, p0 + hi, qe, [](int64_t v, int32_t a) { return v < a; }) - p0;
  j.bytes = kBytesPerPosition * ((int64_t)q->stop - q->start + 1) + kBytesPerRead * (j.re - j.rb);
  if (j.bytes > S->cfg.hbm_budget)
    return serr(S, PG_ERR_NOMEM, "the target needs %lld device bytes, more than the budget of %lld",
                (long long)j.bytes, (long long)S->cfg.hbm_budget);
  j.submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->closing) return serr(S, PG_ERR_STATE, "the server is closing");
    *ticket = S->next_ticket++;
    S->jobs.emplace(*ticket, std::move(j));
    S->queue.push_back(*ticket);
  }
  S->cv_work.notify_one();
  return PG_OK;
} PG_HOST_CATCH(S)

pg_status pg_serve_poll(pg_server* S, uint64_t ticket, int32_t wait_ms, pg_result* out) try {
  if (!S || !out) return PG_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->jobs.find(ticket);
  if (it == S->jobs.end()) return serr(S, PG_ERR_ARG, "unknown ticket %llu", (unsigned long long)ticket);
  Job& j = it->second;
  if (!j.done) {
    if (wait_ms < 0) S->cv_done.wait(lk, [&] { return j.done; });
    else if (wait_ms > 0) S->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return j.done; });
    if (!j.done) return PG_ERR_STATE;  // not answered yet
  }
  auto ms = [](Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
  };
  memset(out, 0, sizeof *out);
  out->status = j.status;
  out->batch = j.batch;
  out->fasta = j.fasta.data();
  out->fasta_len = (int64_t)j.fasta.size();
  out->changes = j.changes.data();
  out->changes_len = (int64_t)j.changes.size();
  out->vcf = j.vcf.data();
  out->vcf_len = (int64_t)j.vcf.size();
  out->message = j.message.c_str();
  out->queue_ms = ms(j.submitted, j.started);
  out->run_ms = ms(j.started, j.finished);
  out->latency_ms = ms(j.submitted, j.finished);
  out->device_bytes = j.bytes;
  return PG_OK;
} PG_HOST_CATCH(S)

pg_status pg_serve_release(pg_server* S, uint64_t ticket) try {
  if (!S) return PG_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->jobs.find(ticket);
  if (it == S->jobs.end()) return serr(S, PG_ERR_ARG, "unknown ticket %llu", (unsigned long long)ticket);
  if (!it->second.done) return serr(S, PG_ERR_STATE, "ticket %llu is not answered yet", (unsigned long long)ticket);
  S->jobs.erase(it);
  return PG_OK;
} PG_HOST_CATCH(S)

pg_status pg_serve_stats(pg_server* S, int64_t* batches, int64_t* in_flight_bytes, int64_t* peak_in_flight_bytes) try {
  if (!S) return PG_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  if (batches) *batches = S->batches;
  if (in_flight_bytes) *in_flight_bytes = S->in_flight;
  if (peak_in_flight_bytes) *peak_in_flight_bytes = S->peak_in_flight;
  return PG_OK;
} PG_HOST_CATCH(S)

const char* pg_serve_error(const pg_server* S) { return S ? S->err.c_str() : "null server"; }

void pg_serve_close(pg_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->closing = true;
  }
  S->cv_work.notify_all();
  for (std::thread& t : S->threads) t.join();
  for (pg_ctx* c : S->workers) pg_close(c);
  if (S->dbuf[0]) {
    cudaSetDevice(S->device);
    free_store(S);
  }
  delete S;
}

}  // extern "C"
