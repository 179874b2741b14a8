// synth.cpp — seeded paired-end read simulator for the benchmark workloads.
//
// Reads are drawn from a sample sequence (the reference with planted SNPs and
// indels) and written as the packed SoA of the C ABI, coordinate-sorted, with
// CIGARs taken from the true alignment of each read to the reference:
//   - sample bases that are planted insertions, sequencing-error insertions or
//     adapter junk align to no reference base; leading/trailing runs of them
//     become soft clips (S), inner runs become insertions (I);
//   - reference bases skipped between two aligned read bases become D;
//   - a pair in which either read keeps fewer than 30 aligned bases is not
//     emitted (a read inside an insertion longer than itself is unmapped, and
//     unmapped reads are left out of the store).
// The random generator is splitmix64 + xoshiro256**, so the output is the same
// on every platform for a given seed.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

namespace {

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    for (int i = 0; i < 4; i++) {
      seed += 0x9E3779B97F4A7C15ull;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      s[i] = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
  }
  double uni() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  int64_t below(int64_t n) { return (int64_t)(uni() * (double)n); }
  double normal() {
    double u1 = uni(), u2 = uni();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

const uint8_t kBaseNib[4] = {1, 2, 4, 8};

inline uint8_t nibOf(uint8_t c) {
  switch (c) {
    case 'A': return 1; case 'C': return 2; case 'G': return 4; case 'T': return 8;
    default: return 15;
  }
}
inline int idxOf(uint8_t c) {
  switch (c) {
    case 'A': return 0; case 'C': return 1; case 'G': return 2; case 'T': return 3;
    default: return 0;
  }
}

struct SimParams {
  int32_t read_len;
  double coverage, insert_mean, insert_sd;
  double sub_err, indel_err, n_frac;
  double mapq0_frac, clip_frac, dup_frac, secondary_frac, improper_frac, noqual_frac;
  int32_t ref_id;
  int32_t repeat_mapq_max;  // reads touching a repeat-masked base get mapq 0..max
};

struct Read {
  int32_t pos, aend, tlen;
  uint16_t flag;
  uint8_t mapq;
  uint32_t cig_begin, cig_n;
  uint64_t base_begin;  // into the bases/quals staging arrays
};

struct Sim {
  std::vector<Read> reads;
  std::vector<uint32_t> cig;
  std::vector<uint8_t> bases, quals;  // ASCII bases and Phred quals, read_len per read
  // outputs (sorted)
  std::vector<int32_t> pos, aend, tlen, refid;
  std::vector<uint16_t> flag, ncig;
  std::vector<uint8_t> mapq, seq, qual;
  std::vector<uint32_t> cigar;
  std::vector<int64_t> cigoff, seqoff, qualoff;
  std::vector<int32_t> lseq;
  std::vector<int64_t> pair;  // the pair each read belongs to (the two mates share a read name)
};

uint8_t drawQual(Rng& r) {
  double q = 40.0 - std::floor(-5.0 * std::log(std::max(r.uni(), 1e-12)));
  if (q < 2) q = 2;
  return (uint8_t)q;
}

// Simulates one read starting at sample position s; returns false if unusable.
bool simRead(Rng& rng, const uint8_t* sample, int64_t slen, const int64_t* s2r, int64_t s, const SimParams& P,
             Sim& S, Read& out, const uint8_t* rmask, int64_t rlen, bool& inRepeat) {
  const int L = P.read_len;
  std::vector<int64_t> r2s(L);  // sample position, -2 error insertion, -3 junk
  double pie = 1.0 - std::pow(1.0 - P.indel_err, L);
  int errK = -1, errType = 0;
  if (rng.uni() < pie) { errK = 15 + (int)rng.below(L - 30); errType = rng.uni() < 0.5 ? 1 : 2; }
  int64_t sp = s;
  for (int k = 0; k < L; k++) {
    if (k == errK && errType == 1) { r2s[k] = -2; continue; }
    if (k == errK && errType == 2) sp++;
    r2s[k] = (sp >= 0 && sp < slen) ? sp : -3;
    sp++;
  }
  if (rng.uni() < P.clip_frac) {
    int c = 5 + (int)rng.below(26);
    if (rng.uni() < 0.5) for (int k = 0; k < c; k++) r2s[k] = -3;
    else for (int k = L - c; k < L; k++) r2s[k] = -3;
  }
  std::vector<int64_t> rref(L);
  int first = -1, last = -1;
  for (int k = 0; k < L; k++) {
    rref[k] = r2s[k] >= 0 ? s2r[r2s[k]] : -1;
    if (rref[k] >= 0) { if (first < 0) first = k; last = k; }
  }
  int mapped = 0;
  for (int k = 0; k < L; k++) mapped += rref[k] >= 0;
  if (mapped < 30) return false;
  // CIGAR
  uint32_t cb = (uint32_t)S.cig.size();
  auto push = [&](int op, int64_t n) {
    if (n <= 0) return;
    if (S.cig.size() > cb && (int)(S.cig.back() & 15) == op) S.cig.back() += (uint32_t)(n << 4);
    else S.cig.push_back((uint32_t)(n << 4) | (uint32_t)op);
  };
  push(4, first);
  int64_t prevRef = -1;
  for (int k = first; k <= last; k++) {
    if (rref[k] < 0) { push(1, 1); continue; }
    if (prevRef >= 0 && rref[k] > prevRef + 1) push(2, rref[k] - prevRef - 1);
    push(0, 1);
    prevRef = rref[k];
  }
  push(4, L - 1 - last);
  out.cig_begin = cb;
  out.cig_n = (uint32_t)(S.cig.size() - cb);
  out.pos = (int32_t)(rref[first] + 1);
  out.aend = (int32_t)(rref[last] + 1);
  inRepeat = false;
  if (rmask) for (int64_t x = rref[first]; x <= rref[last] && x < rlen; x++) if (rmask[x]) { inRepeat = true; break; }
  // bases & quals
  out.base_begin = S.bases.size();
  for (int k = 0; k < L; k++) {
    uint8_t b;
    if (r2s[k] >= 0) b = sample[r2s[k]];
    else b = "ACGT"[rng.below(4)];
    uint8_t q = drawQual(rng);
    if (rng.uni() < P.sub_err) b = "ACGT"[(idxOf(b) + 1 + rng.below(3)) & 3];
    if (rng.uni() < P.n_frac) { b = 'N'; q = 2; }
    S.bases.push_back(b);
    S.quals.push_back(q);
  }
  return true;
}

// Simulates `count` pairs of one contig into S with rng.
static void simPairs(Rng& rng, int64_t count, const uint8_t* sample, int64_t slen, const int64_t* s2r,
                     const uint8_t* repeat_mask, int64_t ref_len, const SimParams* P, Sim* S) {
  const int L = P->read_len;
  S->reads.reserve(2 * count);
  S->bases.reserve((size_t)(2 * count * L));
  S->quals.reserve((size_t)(2 * count * L));
  for (int64_t p = 0; p < count; p++) {
    int64_t fl = (int64_t)std::llround(P->insert_mean + P->insert_sd * rng.normal());
    fl = std::max<int64_t>(fl, L);
    fl = std::min<int64_t>(fl, slen);
    int64_t fs = rng.below(slen - fl + 1);
    size_t mark = S->reads.size(), cmark = S->cig.size(), bmark = S->bases.size();
    Read a{}, b{};
    bool ra = false, rb = false;
    bool okA = simRead(rng, sample, slen, s2r, fs, *P, *S, a, repeat_mask, ref_len, ra);
    bool okB = okA && simRead(rng, sample, slen, s2r, fs + fl - L, *P, *S, b, repeat_mask, ref_len, rb);
    double u1 = rng.uni(), u2 = rng.uni(), u3 = rng.uni(), u4 = rng.uni(), u5 = rng.uni(), u6 = rng.uni();
    if (!(okA && okB)) {
      S->reads.resize(mark); S->cig.resize(cmark); S->bases.resize(bmark); S->quals.resize(bmark);
      continue;
    }
    uint8_t mq = u1 < P->mapq0_frac ? 0 : 60;
    uint8_t mqa = mq, mqb = mq;
    if (P->repeat_mapq_max >= 0) {
      if (ra) mqa = (uint8_t)(rng.below(P->repeat_mapq_max + 1));
      if (rb) mqb = (uint8_t)(rng.below(P->repeat_mapq_max + 1));
    }
    bool proper = u2 >= P->improper_frac;
    bool dup = u3 < P->dup_frac;
    bool aFirst = u4 < 0.5;
    uint16_t base = 0x1 | (proper ? 0x2 : 0) | (dup ? 0x400 : 0);
    a.flag = base | 0x20 | (aFirst ? 0x40 : 0x80);
    b.flag = base | 0x10 | (aFirst ? 0x80 : 0x40);
    if (u5 < P->secondary_frac) a.flag |= 0x100;
    a.mapq = mqa; b.mapq = mqb;
    int32_t left = std::min(a.pos, b.pos), right = std::max(a.aend, b.aend);
    int32_t t = right - left + 1;
    if (a.pos <= b.pos) { a.tlen = t; b.tlen = -t; } else { a.tlen = -t; b.tlen = t; }
    S->reads.push_back(a);
    S->reads.push_back(b);
    if (u6 < P->noqual_frac) {
      for (int k = 0; k < L; k++) S->quals[a.base_begin + k] = 0xFF;
    }
  }
}

}  // namespace

extern "C" {

// Simulates pairs over one contig.  Returns a handle; read sizes with
// sy_n_reads / sy_n_cigar, copy out with sy_copy, free with sy_free.
// Pairs are drawn in blocks of kPairBlock: block 0 from the contig's seed,
// block b from a seed derived from (seed, b); blocks run on parallel threads
// and the result does not depend on the thread count.
void* sy_simulate(const uint8_t* sample, int64_t slen, const int64_t* s2r, const uint8_t* repeat_mask, int64_t ref_len,
                  const SimParams* P, uint64_t seed) {
  constexpr int64_t kPairBlock = 1000000;
  Sim* S = new Sim();
  const int L = P->read_len;
  const int64_t nPairs = (int64_t)std::llround(P->coverage * (double)slen / (2.0 * L));
  const int64_t nb = std::max<int64_t>(1, (nPairs + kPairBlock - 1) / kPairBlock);
  if (nb == 1) {
    Rng rng(seed);
    simPairs(rng, nPairs, sample, slen, s2r, repeat_mask, ref_len, P, S);
  } else {
    std::vector<Sim> parts((size_t)nb);
    std::atomic<int64_t> next{0};
    auto work = [&]() {
      for (int64_t b; (b = next.fetch_add(1)) < nb;) {
        Rng rng(b == 0 ? seed : seed ^ (0xD1B54A32D192ED03ull * (uint64_t)(b + 1)));
        simPairs(rng, std::min(kPairBlock, nPairs - b * kPairBlock), sample, slen, s2r, repeat_mask, ref_len, P,
                 &parts[(size_t)b]);
      }
    };
    const int64_t nt = std::min<int64_t>(nb, std::max(1u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int64_t k = 1; k < nt; k++) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
    for (Sim& q : parts) {  // concatenate the blocks in order
      const uint32_t c0 = (uint32_t)S->cig.size();
      const uint64_t b0 = S->bases.size();
      for (Read r : q.reads) {
        r.cig_begin += c0;
        r.base_begin += b0;
        S->reads.push_back(r);
      }
      S->cig.insert(S->cig.end(), q.cig.begin(), q.cig.end());
      S->bases.insert(S->bases.end(), q.bases.begin(), q.bases.end());
      S->quals.insert(S->quals.end(), q.quals.begin(), q.quals.end());
      std::vector<Read>().swap(q.reads);
      std::vector<uint32_t>().swap(q.cig);
      std::vector<uint8_t>().swap(q.bases);
      std::vector<uint8_t>().swap(q.quals);
    }
  }
  // sort by position (stable)
  std::vector<uint32_t> order(S->reads.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return S->reads[x].pos < S->reads[y].pos; });
  size_t n = order.size();
  S->pos.resize(n); S->aend.resize(n); S->tlen.resize(n); S->refid.assign(n, P->ref_id);
  S->flag.resize(n); S->ncig.resize(n); S->mapq.resize(n); S->lseq.assign(n, L);
  S->cigoff.resize(n); S->seqoff.resize(n); S->qualoff.resize(n); S->pair.resize(n);
  S->seq.resize(n * (size_t)((L + 1) / 2));
  S->qual.resize(n * (size_t)L);
  S->cigar.reserve(S->cig.size());
  for (size_t i = 0; i < n; i++) {
    const Read& r = S->reads[order[i]];
    S->pair[i] = (int64_t)(order[i] >> 1);  // mates are pushed one after the other
    S->pos[i] = r.pos; S->aend[i] = r.aend; S->tlen[i] = r.tlen; S->flag[i] = r.flag; S->mapq[i] = r.mapq;
    S->cigoff[i] = (int64_t)S->cigar.size();
    S->ncig[i] = (uint16_t)r.cig_n;
    for (uint32_t k = 0; k < r.cig_n; k++) S->cigar.push_back(S->cig[r.cig_begin + k]);
    S->seqoff[i] = (int64_t)(i * (size_t)((L + 1) / 2));
    S->qualoff[i] = (int64_t)(i * (size_t)L);
    uint8_t* sq = &S->seq[S->seqoff[i]];
    for (int k = 0; k < L; k += 2) {
      uint8_t hi = nibOf(S->bases[r.base_begin + k]);
      uint8_t lo = k + 1 < L ? nibOf(S->bases[r.base_begin + k + 1]) : 0;
      sq[k / 2] = (uint8_t)((hi << 4) | lo);
    }
    memcpy(&S->qual[S->qualoff[i]], &S->quals[r.base_begin], L);
  }
  std::vector<Read>().swap(S->reads);
  std::vector<uint32_t>().swap(S->cig);
  std::vector<uint8_t>().swap(S->bases);
  std::vector<uint8_t>().swap(S->quals);
  return S;
}

int64_t sy_n_reads(void* h) { return (int64_t)((Sim*)h)->pos.size(); }
int64_t sy_n_cigar(void* h) { return (int64_t)((Sim*)h)->cigar.size(); }

void sy_copy(void* h, int32_t* pos, int32_t* aend, uint16_t* flag, uint8_t* mapq, int32_t* tlen, int32_t* refid,
             int64_t* cigoff, uint16_t* ncig, uint32_t* cigar, int64_t* seqoff, int32_t* lseq, uint8_t* seq,
             int64_t* qualoff, uint8_t* qual) {
  Sim* S = (Sim*)h;
  size_t n = S->pos.size();
  memcpy(pos, S->pos.data(), n * 4); memcpy(aend, S->aend.data(), n * 4); memcpy(flag, S->flag.data(), n * 2);
  memcpy(mapq, S->mapq.data(), n); memcpy(tlen, S->tlen.data(), n * 4); memcpy(refid, S->refid.data(), n * 4);
  memcpy(cigoff, S->cigoff.data(), n * 8); memcpy(ncig, S->ncig.data(), n * 2);
  memcpy(cigar, S->cigar.data(), S->cigar.size() * 4);
  memcpy(seqoff, S->seqoff.data(), n * 8); memcpy(lseq, S->lseq.data(), n * 4);
  memcpy(seq, S->seq.data(), S->seq.size()); memcpy(qualoff, S->qualoff.data(), n * 8);
  memcpy(qual, S->qual.data(), S->qual.size());
}

// The pair index of every read (sorted order): mates share it, as they share
// a read name in a BAM.
void sy_copy_pairs(void* h, int64_t* pair) {
  Sim* S = (Sim*)h;
  memcpy(pair, S->pair.data(), S->pair.size() * 8);
}

void sy_free(void* h) { delete (Sim*)h; }

int32_t sy_params_size(void) { return (int32_t)sizeof(SimParams); }

}  // extern "C"
