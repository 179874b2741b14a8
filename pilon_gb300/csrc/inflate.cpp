// inflate.cpp — raw DEFLATE (RFC 1951) decoding of the BGZF blocks of a BAM
// file, the decompression htsjdk's BlockCompressedInputStream does before
// BamFile reads records (S/BamFile.scala:117-126).
//
// Every BGZF block is an independent raw DEFLATE stream with a known output
// size, so the blocks are decoded on worker threads straight into their place
// in one output buffer.  Huffman codes are decoded from a 10-bit lookup table;
// the rare longer codes are finished bit by bit with the canonical code counts.
// Every read of the input and every write of the output is bounds checked: a
// damaged stream ends with an error, never outside its buffers.
#include <atomic>
#include <cstdint>
#include <cstring>
#include <exception>
#include <thread>
#include <vector>

namespace {

constexpr int kMaxBits = 15, kFastBits = 10;

// Length base and extra bits for symbols 257..285, distance base and extra bits
// for codes 0..29 (RFC 1951, 3.2.5).
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// order of the code length code lengths in a dynamic block header
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// Little-endian bit reader over [p, end): bits past the end read as zero and
// are counted, so a decoder that consumed them reports a truncated stream.
// With 8 bytes left a refill loads a whole word: the bytes past the counted
// bits are ORed in again, at the same places, by the next refill.
struct Bits {
  const uint8_t* p;
  const uint8_t* end;
  uint64_t buf = 0;
  int cnt = 0;
  int64_t over = 0;  // bits supplied past the end
  void refill() {
    if (end - p >= 8) {
      uint64_t w;
      std::memcpy(&w, p, 8);
      buf |= w << cnt;
      p += (63 - cnt) >> 3;
      cnt |= 56;
      return;
    }
    while (cnt <= 56) {
      if (p < end) buf |= (uint64_t)*p++ << cnt;
      else over += 8;
      cnt += 8;
    }
  }
  uint32_t peek(int n) {
    if (cnt < n) refill();
    return (uint32_t)(buf & ((1ull << n) - 1));
  }
  void drop(int n) { buf >>= n; cnt -= n; }
  uint32_t take(int n) {
    if (n == 0) return 0;
    const uint32_t v = peek(n);
    drop(n);
    return v;
  }
  // n bits that the caller has already made available
  uint32_t take_have(int n) {
    const uint32_t v = (uint32_t)(buf & ((1ull << n) - 1));
    drop(n);
    return v;
  }
  // the bits consumed past the end: those supplied there minus the ones still held
  bool overrun() const { return over > (int64_t)cnt; }
};

// The alphabets a code is built for, and the kinds of combined entries.
enum Alphabet { kCodeLengths = 0, kLitLen = 1, kDist = 2 };
enum Kind : uint32_t { kSlow = 0, kLiteral = 1, kLength = 2, kEnd = 3, kDistance = 4 };

// A canonical Huffman code: counts and symbols in code order (for the slow
// path) and two 10-bit tables.  fast[] = symbol | length << 16, or 0 when the
// code is longer than 10 bits (or the bits match no code).  entry[] holds what
// the symbol loop needs in one load: the value (literal byte, length or
// distance base) << 16 | kind << 9 | code length << 5 | code length + extra
// bits; kind kSlow sends the loop to the generic path.
struct Huff {
  uint16_t count[kMaxBits + 1];
  uint16_t symbol[320];
  uint32_t fast[1 << kFastBits];
  uint32_t entry[1 << kFastBits];

  static uint32_t combined(int alpha, int sym, int l) {
    uint32_t value = 0, extra = 0, kind = kSlow;
    if (alpha == kLitLen) {
      if (sym < 256) { value = (uint32_t)sym; kind = kLiteral; }
      else if (sym == 256) { kind = kEnd; }
      else if (sym < 286) { value = kLenBase[sym - 257]; extra = kLenExtra[sym - 257]; kind = kLength; }
    } else if (alpha == kDist && sym < 30) {
      value = kDistBase[sym]; extra = kDistExtra[sym]; kind = kDistance;
    }
    return value << 16 | kind << 9 | (uint32_t)l << 5 | ((uint32_t)l + extra);
  }

  // false for an over-subscribed set of lengths; incomplete codes (allowed
  // for a single distance code) decode as long as no missing code is met
  bool build(const uint8_t* len, int n, int alpha = kCodeLengths) {
    std::memset(count, 0, sizeof count);
    for (int s = 0; s < n; s++) count[len[s]]++;
    count[0] = 0;
    int left = 1;
    for (int l = 1; l <= kMaxBits; l++) {
      left <<= 1;
      left -= count[l];
      if (left < 0) return false;
    }
    uint16_t offs[kMaxBits + 2];
    offs[1] = 0;
    for (int l = 1; l <= kMaxBits; l++) offs[l + 1] = offs[l] + count[l];
    for (int s = 0; s < n; s++)
      if (len[s]) symbol[offs[len[s]]++] = (uint16_t)s;
    std::memset(fast, 0, sizeof fast);
    std::memset(entry, 0, sizeof entry);  // kSlow
    // canonical codes in order of length, then symbol
    uint32_t code = 0;
    int idx = 0;
    for (int l = 1; l <= kMaxBits; l++) {
      for (int k = 0; k < count[l]; k++, idx++, code++) {
        if (l > kFastBits) continue;
        uint32_t rev = 0;  // the stream holds the code's bits from its top bit down
        for (int b = 0; b < l; b++) rev |= ((code >> b) & 1u) << (l - 1 - b);
        const uint32_t fe = symbol[idx] | ((uint32_t)l << 16), ce = combined(alpha, symbol[idx], l);
        for (uint32_t f = rev; f < (1u << kFastBits); f += 1u << l) {
          fast[f] = fe;
          entry[f] = ce;
        }
      }
      code <<= 1;
    }
    return true;
  }

  // next symbol, or -1 when the bits match no code
  int decode(Bits& in) const { return decode_bits(in, in.peek(kMaxBits)); }
  // the same when the caller has made 15 bits available
  int decode_have(Bits& in) const { return decode_bits(in, (uint32_t)in.buf & ((1u << kMaxBits) - 1)); }
  int decode_bits(Bits& in, uint32_t v) const {
    const uint32_t e = fast[v & ((1u << kFastBits) - 1)];
    if (e) {
      in.drop((int)(e >> 16));
      return (int)(e & 0xffffu);
    }
    // longer codes: walk the lengths, one more bit of the code each step
    int code = 0, first = 0, index = 0;
    for (int l = 1; l <= kMaxBits; l++) {
      code |= (int)((v >> (l - 1)) & 1u);
      const int c = count[l];
      if (code - c < first) {
        in.drop(l);
        return symbol[index + (code - first)];
      }
      index += c;
      first += c;
      first <<= 1;
      code <<= 1;
    }
    return -1;
  }
};

struct Decoder {
  Huff lit, dist;

  // inflates [src, src + n) into [dst, dst + cap); returns the bytes written
  // or -1 for a damaged stream
  int64_t run(const uint8_t* src, int64_t n, uint8_t* dst, int64_t cap) {
    Bits in{src, src + n};
    int64_t o = 0;
    bool last = false;
    while (!last) {
      last = in.take(1) != 0;
      const uint32_t type = in.take(2);
      if (type == 0) {  // stored: to the byte boundary, LEN, NLEN, LEN bytes
        in.drop(in.cnt & 7);
        const uint32_t len = in.take(16), nlen = in.take(16);
        if ((len ^ 0xffffu) != nlen) return -1;
        for (uint32_t k = 0; k < len; k++) {
          if (o >= cap) return -1;
          dst[o++] = (uint8_t)in.take(8);
        }
        if (in.overrun()) return -1;
        continue;
      }
      if (type == 3) return -1;
      if (type == 1) {
        uint8_t l[320];
        for (int s = 0; s < 144; s++) l[s] = 8;
        for (int s = 144; s < 256; s++) l[s] = 9;
        for (int s = 256; s < 280; s++) l[s] = 7;
        for (int s = 280; s < 288; s++) l[s] = 8;
        lit.build(l, 288, kLitLen);
        for (int s = 0; s < 30; s++) l[s] = 5;
        dist.build(l, 30, kDist);
      } else if (!read_tables(in)) {
        return -1;
      }
      // Symbols until end of block, from the combined entries: a literal, a
      // length or a distance with its extra bits in one load and one shift.
      // One refill gives the bits of two literals and a length (10 + 10 + 20
      // <= 48); the distance (15 + 13) refills if needed.  Codes longer than
      // the table take the generic path.  Bits read past the end of the input
      // are zeros; every pass emits output (bounded by cap), ends the block
      // or fails, so the overrun is checked per block.
      constexpr uint32_t kMask = (1u << kFastBits) - 1;
      // the bit reader's state in locals (registers) for the loop; it is
      // written back around the generic path and at the end of the block
      uint64_t bb = in.buf;
      int bc = in.cnt;
      const uint8_t* ip = in.p;
      int64_t over = in.over;
      const uint8_t* const iend = in.end;
      auto need = [&](int nb) {
        if (bc >= nb) return;
        if (iend - ip >= 8) {
          uint64_t w;
          std::memcpy(&w, ip, 8);
          bb |= w << bc;
          ip += (63 - bc) >> 3;
          bc |= 56;
        } else {
          while (bc <= 56) {
            if (ip < iend) bb |= (uint64_t)*ip++ << bc;
            else over += 8;
            bc += 8;
          }
        }
      };
      auto drop = [&](int nb) {
        bb >>= nb;
        bc -= nb;
      };
      auto store = [&]() {
        in.buf = bb;
        in.cnt = bc;
        in.p = ip;
        in.over = over;
      };
      auto load = [&]() {
        bb = in.buf;
        bc = in.cnt;
        ip = in.p;
        over = in.over;
      };
      while (true) {
        need(48);
        uint32_t e = lit.entry[bb & kMask];
        if ((e >> 9 & 7) == kLiteral) {
          drop((int)(e & 31));
          if (o >= cap) return -1;
          dst[o++] = (uint8_t)(e >> 16);
          e = lit.entry[bb & kMask];
          if ((e >> 9 & 7) == kLiteral) {
            drop((int)(e & 31));
            if (o >= cap) return -1;
            dst[o++] = (uint8_t)(e >> 16);
            continue;
          }
        }
        int64_t len;
        const uint32_t kind = e >> 9 & 7;
        if (kind == kLength) {
          const uint32_t cl = e >> 5 & 15, tot = e & 31;
          len = (int64_t)(e >> 16) + (int64_t)((bb >> cl) & ((1ull << (tot - cl)) - 1));
          drop((int)tot);
        } else if (kind == kEnd) {
          drop((int)(e & 31));
          break;
        } else {  // a code longer than the table, or no code: >= 38 bits remain
          store();
          const int sym = lit.decode_have(in);
          int li = -1;
          if (sym >= 257) {
            li = sym - 257;
            if (li < 29) len = kLenBase[li] + in.take_have(kLenExtra[li]);
          }
          load();
          if (sym < 0) return -1;
          if (sym < 256) {
            if (o >= cap) return -1;
            dst[o++] = (uint8_t)sym;
            continue;
          }
          if (sym == 256) break;
          if (li >= 29) return -1;
        }
        {
          need(28);
          const uint32_t de = dist.entry[bb & kMask];
          int64_t d;
          if ((de >> 9 & 7) == kDistance) {
            const uint32_t cl = de >> 5 & 15, tot = de & 31;
            d = (int64_t)(de >> 16) + (int64_t)((bb >> cl) & ((1ull << (tot - cl)) - 1));
            drop((int)tot);
          } else {
            store();
            const int ds = dist.decode_have(in);
            d = (ds >= 0 && ds < 30) ? kDistBase[ds] + in.take_have(kDistExtra[ds]) : -1;
            load();
            if (d < 0) return -1;
          }
          if (d > o || len > cap - o) return -1;
          uint8_t* w = dst + o;
          const uint8_t* r = w - d;
          if (d >= 8 && cap - o >= len + 8) {
            // 8 bytes at a time: each source word lies at least 8 bytes behind its
            // destination, so overlapping matches repeat their pattern correctly;
            // the last word may write up to 7 bytes past the match, inside dst
            for (int64_t k = 0; k < len; k += 8) {
              uint64_t v;
              std::memcpy(&v, r + k, 8);
              std::memcpy(w + k, &v, 8);
            }
          } else if (d == 1) {
            std::memset(w, *r, (size_t)len);
          } else if (d >= len) {
            std::memcpy(w, r, (size_t)len);
          } else {
            for (int64_t k = 0; k < len; k++) w[k] = r[k];  // overlapping copy repeats the pattern
          }
          o += len;
        }
      }
      store();
      if (in.overrun()) return -1;
    }
    return o;
  }

  bool read_tables(Bits& in) {
    const int hlit = (int)in.take(5) + 257, hdist = (int)in.take(5) + 1, hclen = (int)in.take(4) + 4;
    if (hlit > 286 || hdist > 30) return false;
    uint8_t cl[19] = {0};
    for (int k = 0; k < hclen; k++) cl[kClOrder[k]] = (uint8_t)in.take(3);
    Huff clh;
    if (!clh.build(cl, 19)) return false;
    uint8_t lens[320];
    int k = 0;
    while (k < hlit + hdist) {
      const int sym = clh.decode(in);
      if (sym < 0) return false;
      if (sym < 16) {
        lens[k++] = (uint8_t)sym;
        continue;
      }
      int rep;
      uint8_t v = 0;
      if (sym == 16) {
        if (k == 0) return false;
        v = lens[k - 1];
        rep = 3 + (int)in.take(2);
      } else if (sym == 17) {
        rep = 3 + (int)in.take(3);
      } else {
        rep = 11 + (int)in.take(7);
      }
      if (k + rep > hlit + hdist) return false;
      while (rep--) lens[k++] = v;
    }
    if (in.overrun() || lens[256] == 0) return false;  // no end-of-block code
    return lit.build(lens, hlit, kLitLen) && dist.build(lens + hlit, hdist, kDist);
  }
};

}  // namespace

extern "C" {

// The BGZF blocks of a file (SAM/BAM specification 4.1): gzip members with
// FEXTRA and a BC subfield holding the block size.  Writes each block's
// compressed data [src_off, src_end) and its uncompressed size (at most
// 64 KiB); cap entries suffice when cap >= n / 28 + 1, a block taking at least
// 28 bytes.  Returns the block count, or -1 with *err_off the block's offset
// and *err_kind 1 (not a BGZF block), 2 (truncated), 3 (no BC subfield),
// 4 (more than 64 KiB uncompressed) or 5 (more blocks than cap).
int64_t bgzf_scan(const uint8_t* raw, int64_t n, int64_t* src_off, int64_t* src_end, int64_t* out_size, int64_t cap,
                  int64_t* err_off, int32_t* err_kind) {
  int64_t off = 0, k = 0;
  auto fail = [&](int32_t kind) {
    *err_off = off;
    *err_kind = kind;
    return (int64_t)-1;
  };
  while (off < n) {
    if (off + 18 > n || raw[off] != 0x1F || raw[off + 1] != 0x8B || (raw[off + 3] & 4) == 0) return fail(1);
    const int64_t xlen = raw[off + 10] | (int64_t)raw[off + 11] << 8;
    if (off + 12 + xlen > n) return fail(2);
    int64_t x = off + 12, bsize = -1;
    while (x + 4 <= off + 12 + xlen) {
      const int64_t slen = raw[x + 2] | (int64_t)raw[x + 3] << 8;
      if (raw[x] == 66 && raw[x + 1] == 67 && slen == 2 && x + 6 <= off + 12 + xlen)
        bsize = raw[x + 4] | (int64_t)raw[x + 5] << 8;
      x += 4 + slen;
    }
    if (bsize < 0) return fail(3);
    const int64_t end = off + bsize + 1;
    if (end > n || end - 8 < off + 12 + xlen) return fail(2);
    const int64_t isize = raw[end - 4] | (int64_t)raw[end - 3] << 8 | (int64_t)raw[end - 2] << 16 |
                          (int64_t)raw[end - 1] << 24;
    if (isize > 65536) return fail(4);
    if (k >= cap) return fail(5);
    src_off[k] = off + 12 + xlen;
    src_end[k] = end - 8;
    out_size[k] = isize;
    k++;
    off = end;
  }
  return k;
}

// Inflates n_blocks raw DEFLATE streams: block k is in[src_off[k], src_end[k])
// of `in` and must produce exactly out_size[k] bytes at out + out_off[k].
// Returns 0, or -(k + 1) for the first damaged block found.
int64_t bgzf_inflate_blocks(const uint8_t* in, int64_t n_blocks, const int64_t* src_off, const int64_t* src_end,
                            const int64_t* out_off, const int64_t* out_size, uint8_t* out, int32_t threads) {
  std::atomic<int64_t> next{0}, bad{-1};
  auto work = [&]() {
    Decoder dec;
    while (true) {
      const int64_t k = next.fetch_add(1);
      if (k >= n_blocks) break;
      if (out_size[k] == 0) continue;
      const int64_t got = dec.run(in + src_off[k], src_end[k] - src_off[k], out + out_off[k], out_size[k]);
      if (got != out_size[k]) {
        int64_t cur = bad.load();
        while ((cur < 0 || k < cur) && !bad.compare_exchange_weak(cur, k)) {}
      }
    }
  };
  const int nt = threads < 1 ? 1 : threads;
  std::vector<std::thread> pool;
  try {  // blocks are taken from a shared counter: threads that cannot start leave them to the others
    pool.reserve((size_t)nt);
    for (int t = 1; t < nt; t++) pool.emplace_back(work);
  } catch (const std::exception&) {
  }
  work();
  for (auto& t : pool) t.join();
  return bad.load() < 0 ? 0 : -(bad.load() + 1);
}

}  // extern "C"
