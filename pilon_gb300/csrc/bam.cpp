// bam.cpp — BAM records <-> the packed read store of the C ABI (pg_reads).
//
// The host side of BamFile's input (S/BamFile.scala:117-126, htsjdk's
// SAMRecord decoding): the caller inflates the BGZF blocks (inflate.cpp does it
// on parallel threads) and passes the decompressed stream after the header;
// these functions split it into records and fill the structure-of-arrays
// store, or encode a store as BAM records.
//
// Record layout (SAM/BAM specification 4.2): block_size, refID, pos (0-based),
// l_read_name, mapq, bin, n_cigar_op, flag, l_seq, next_refID, next_pos, tlen,
// read_name, cigar (len << 4 | op), seq (4-bit), qual (0xFF when absent), tags.
// The store keeps BAM's CIGAR words, nibbles and qualities unchanged; pos is
// 1-based (htsjdk getAlignmentStart) and aend is htsjdk getAlignmentEnd: the
// start plus the reference length of the CIGAR minus one, 0 for an unmapped read.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <exception>
#include <thread>
#include <string_view>
#include <unordered_map>
#include <vector>

namespace {

inline int32_t rd32(const uint8_t* p) {
  int32_t v;
  std::memcpy(&v, p, 4);
  return v;
}
inline uint16_t rd16(const uint8_t* p) {
  uint16_t v;
  std::memcpy(&v, p, 2);
  return v;
}
inline void wr32(uint8_t* p, int32_t v) { std::memcpy(p, &v, 4); }
inline void wr16(uint8_t* p, uint16_t v) { std::memcpy(p, &v, 2); }

inline bool consumes_ref(uint32_t op) { return op == 0 || op == 2 || op == 3 || op == 7 || op == 8; }

// reg2bin of the BAM specification (section 5.3), 0-based [beg, end)
inline uint16_t reg2bin(int32_t beg, int32_t end) {
  --end;
  if (beg >> 14 == end >> 14) return (uint16_t)(((1 << 15) - 1) / 7 + (beg >> 14));
  if (beg >> 17 == end >> 17) return (uint16_t)(((1 << 12) - 1) / 7 + (beg >> 17));
  if (beg >> 20 == end >> 20) return (uint16_t)(((1 << 9) - 1) / 7 + (beg >> 20));
  if (beg >> 23 == end >> 23) return (uint16_t)(((1 << 6) - 1) / 7 + (beg >> 23));
  if (beg >> 26 == end >> 26) return (uint16_t)(((1 << 3) - 1) / 7 + (beg >> 26));
  return 0;
}

}  // namespace

extern "C" {

// One walk of the record chain of a decompressed record stream: checks that
// every record fits its block_size and the stream, writes each record's offset
// to starts (cap entries; a record takes at least 36 bytes, so n / 36 + 1
// always suffice) and the sizes of the store's variable arrays.  Returns the
// record count, or -1 - offset of the first record that does not fit.
int64_t bam_index(const uint8_t* buf, int64_t n, int64_t* starts, int64_t cap, int64_t* n_cigar, int64_t* seq_bytes,
                  int64_t* qual_bytes) {
  int64_t off = 0, recs = 0, nc = 0, sb = 0, qb = 0;
  while (off + 4 <= n) {
    const int32_t bs = rd32(buf + off);
    if (bs < 32 || off + 4 + bs > n) return -1 - off;
    const uint8_t* r = buf + off + 4;
    const int32_t l_seq = rd32(r + 16);
    const uint32_t l_name = r[8], n_cig = rd16(r + 12);
    if (l_seq < 0 || 32 + (int64_t)l_name + 4 * (int64_t)n_cig + ((int64_t)l_seq + 1) / 2 + l_seq > bs)
      return -1 - off;
    if (recs >= cap) return -1 - off;
    starts[recs++] = off;
    nc += n_cig;
    sb += ((int64_t)l_seq + 1) / 2;
    qb += l_seq;
    off += 4 + bs;
  }
  if (off != n) return -1 - off;
  *n_cigar = nc;
  *seq_bytes = sb;
  *qual_bytes = qb;
  return recs;
}

// Fills the store (arrays sized by bam_index) from the records at starts, on
// `threads` threads over contiguous ranges of records: each thread first sums
// its records' CIGAR words, base bytes and qualities, and after a prefix over
// the threads fills its range from its own offsets.  Returns the record count,
// or -1 when host memory runs out (threads that cannot be started leave their
// ranges to the calling thread).
int64_t bam_fill(const uint8_t* buf, const int64_t* starts, int64_t recs, int32_t* pos, int32_t* aend, int32_t* tlen,
                 int32_t* ref_id, int32_t* mate_ref_id, int32_t* l_seq_out, uint16_t* flag, uint16_t* n_cigar,
                 uint8_t* mapq, uint8_t* seq, uint8_t* qual, int64_t* cigar_off, int64_t* seq_off, int64_t* qual_off,
                 uint32_t* cigar, int32_t threads) try {
  const int64_t nt = std::max<int64_t>(1, std::min<int64_t>(threads < 1 ? 1 : threads, recs));
  std::vector<int64_t> tc(nt + 1, 0), ts(nt + 1, 0), tq(nt + 1, 0);
  auto lo = [&](int64_t t) { return recs * t / nt; };
  auto run = [&](auto&& body) {
    std::vector<std::thread> pool;
    int64_t t = 1;
    try {
      pool.reserve((size_t)nt);
      for (; t < nt; t++) pool.emplace_back(body, t);
    } catch (const std::exception&) {
    }
    for (int64_t u = t; u < nt; u++) body(u);
    body(0);
    for (auto& th : pool) th.join();
  };
  run([&](int64_t t) {
    int64_t c = 0, sb = 0, qb = 0;
    for (int64_t i = lo(t); i < lo(t + 1); i++) {
      const uint8_t* r = buf + starts[i] + 4;
      const int32_t ls = rd32(r + 16);
      c += rd16(r + 12);
      sb += ((int64_t)ls + 1) / 2;
      qb += ls;
    }
    tc[t + 1] = c;
    ts[t + 1] = sb;
    tq[t + 1] = qb;
  });
  for (int64_t t = 0; t < nt; t++) {
    tc[t + 1] += tc[t];
    ts[t + 1] += ts[t];
    tq[t + 1] += tq[t];
  }
  run([&](int64_t t) {
    int64_t co = tc[t], so = ts[t], qo = tq[t];
    for (int64_t i = lo(t); i < lo(t + 1); i++) {
      const uint8_t* r = buf + starts[i] + 4;
      const int32_t rid = rd32(r), p0 = rd32(r + 4);
      const uint32_t l_name = r[8];
      const uint16_t nc = rd16(r + 12), fl = rd16(r + 14);
      const int32_t ls = rd32(r + 16);
      const uint8_t* cg = r + 32 + l_name;
      const uint8_t* sq = cg + 4 * (int64_t)nc;
      const uint8_t* ql = sq + ((int64_t)ls + 1) / 2;
      int64_t reflen = 0;
      for (uint32_t k = 0; k < nc; k++) {
        uint32_t w;
        std::memcpy(&w, cg + 4 * k, 4);
        cigar[co + k] = w;
        if (consumes_ref(w & 15u)) reflen += w >> 4;
      }
      pos[i] = (int32_t)((uint32_t)p0 + 1u);  // Java int arithmetic: wraps
      aend[i] = (fl & 0x4) ? 0 : (int32_t)(p0 + reflen);  // (p0 + 1) + reflen - 1
      tlen[i] = rd32(r + 28);
      ref_id[i] = rid;
      mate_ref_id[i] = rd32(r + 20);
      l_seq_out[i] = ls;
      flag[i] = fl;
      n_cigar[i] = nc;
      mapq[i] = r[9];
      cigar_off[i] = co;
      seq_off[i] = so;
      qual_off[i] = qo;
      std::memcpy(seq + so, sq, (size_t)(((int64_t)ls + 1) / 2));
      std::memcpy(qual + qo, ql, (size_t)ls);
      co += nc;
      so += ((int64_t)ls + 1) / 2;
      qo += ls;
    }
  });
  return recs;
} catch (const std::exception&) {
  return -1;
}

// The read name of read i: "p<name_id[i]>" (mates share it) or, without name
// ids, "r<i>"; returns its length with the NUL.
static int read_name(char* name, size_t cap, const int64_t* name_id, int64_t i) {
  return (name_id ? std::snprintf(name, cap, "p%lld", (long long)name_id[i])
                  : std::snprintf(name, cap, "r%lld", (long long)i)) + 1;
}

// Read-name ids of the records at starts: the first record with a name gets
// the next id, later records with the same name (mates, other alignments) its
// id, as htsjdk's getReadName strings compare.  Single pass, exact.  Returns
// the number of distinct names, or -1 when host memory runs out.
int64_t bam_name_ids(const uint8_t* buf, const int64_t* starts, int64_t recs, int64_t* out) try {
  std::unordered_map<std::string_view, int64_t> ids;
  ids.reserve((size_t)(recs / 2 + 1));
  for (int64_t i = 0; i < recs; i++) {
    const uint8_t* r = buf + starts[i] + 4;
    const uint32_t l_name = r[8];
    const char* nm = reinterpret_cast<const char*>(r + 32);
    const size_t len = l_name > 0 ? strnlen(nm, l_name) : 0;  // up to the NUL
    auto it = ids.emplace(std::string_view(nm, len), (int64_t)ids.size()).first;
    out[i] = it->second;
  }
  return (int64_t)ids.size();
} catch (const std::exception&) {
  return -1;
}

// Bytes of the BAM records of reads [0, n) (read names as read_name gives them).
int64_t bam_encoded_size(int64_t n, const uint16_t* n_cigar, const int32_t* l_seq, const int64_t* name_id) {
  int64_t total = 0;
  char name[32];
  for (int64_t i = 0; i < n; i++) {
    const int ln = read_name(name, sizeof name, name_id, i);
    total += 4 + 32 + ln + 4 * (int64_t)n_cigar[i] + (l_seq[i] + 1) / 2 + l_seq[i];
  }
  return total;
}

// Encodes reads [0, n) of a store as BAM records into out (bam_encoded_size
// bytes).  Returns the bytes written.
int64_t bam_encode(int64_t n, const int32_t* pos, const int32_t* tlen, const int32_t* ref_id,
                   const int32_t* mate_ref_id, const int32_t* l_seq, const uint16_t* flag, const uint16_t* n_cigar,
                   const uint8_t* mapq, const uint8_t* seq, const uint8_t* qual, const int64_t* cigar_off,
                   const int64_t* seq_off, const int64_t* qual_off, const uint32_t* cigar,
                   const int32_t* mate_pos, const int64_t* name_id, uint8_t* out) {
  int64_t o = 0;
  char name[32];
  for (int64_t i = 0; i < n; i++) {
    const int ln = read_name(name, sizeof name, name_id, i);
    const int32_t ls = l_seq[i];
    const uint16_t nc = n_cigar[i];
    const int32_t bs = 32 + ln + 4 * nc + (ls + 1) / 2 + ls;
    uint8_t* r = out + o;
    wr32(r, bs);
    r += 4;
    int64_t reflen = 0;
    for (uint16_t k = 0; k < nc; k++)
      if (consumes_ref(cigar[cigar_off[i] + k] & 15u)) reflen += cigar[cigar_off[i] + k] >> 4;
    const int32_t p0 = pos[i] - 1;
    wr32(r, ref_id[i]);
    wr32(r + 4, p0);
    r[8] = (uint8_t)ln;
    r[9] = mapq[i];
    wr16(r + 10, reg2bin(p0, (int32_t)(p0 + (reflen > 0 ? reflen : 1))));
    wr16(r + 12, nc);
    wr16(r + 14, flag[i]);
    wr32(r + 16, ls);
    wr32(r + 20, mate_ref_id[i]);
    wr32(r + 24, mate_pos ? mate_pos[i] - 1 : -1);
    wr32(r + 28, tlen[i]);
    std::memcpy(r + 32, name, (size_t)ln);
    uint8_t* p = r + 32 + ln;
    std::memcpy(p, cigar + cigar_off[i], 4 * (size_t)nc);
    p += 4 * nc;
    std::memcpy(p, seq + seq_off[i], (size_t)(ls + 1) / 2);
    p += (ls + 1) / 2;
    std::memcpy(p, qual + qual_off[i], (size_t)ls);
    o += 4 + bs;
  }
  return o;
}

}  // extern "C"
