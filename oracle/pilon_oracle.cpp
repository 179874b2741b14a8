// pilon_oracle.cpp — CPU oracle for the pilon_gb300 engine.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, line by line, the Scala code
// of Pilon 1.24 (broadinstitute/pilon) that the GPU engine replaces, so that
// tests and the CPU baseline of bench.py can check the engine against it.  No
// product code links, loads or calls it.
//
// Parity is unpinned by reference tests: the reference ships no tests, golden
// files or known-answer vectors, and no JVM exists here to run it.  The oracle
// is pinned instead by hand-derived known-answer cases (tests/golden/).
//
// Citations are file:line into the reference, S/ = src/main/scala/org/broadinstitute/pilon/.
// Java integer semantics: Scala Int arithmetic wraps at 32 bits; this file is
// compiled with -fwrapv so that signed int32 arithmetic wraps the same way.

#include "../include/pilon_gb300.h"

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <map>
#include <memory>
#include <thread>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

struct IndexError : std::runtime_error {
  IndexError() : std::runtime_error("ArrayIndexOutOfBounds") {}
};

const char kNib[] = "=ACMGRSVTWYHKDBN";

// S/Utils.scala:23-26
inline int64_t roundDivL(int64_t n, int64_t d) { return d > 0 ? (n + d / 2) / d : 0; }
inline int32_t roundDivI(int32_t n, int32_t d) { return d > 0 ? (n + d / 2) / d : 0; }
inline int64_t pctL(int64_t n, int64_t d) { return roundDivL(100 * n, d); }
inline int32_t pctI(int32_t n, int32_t d) { return roundDivI(100 * n, d); }

// java.lang.Math.round(double): nearest, ties toward positive infinity; NaN
// gives 0 and values beyond the long range saturate (JLS 5.1.3).
inline int64_t javaRound(double x) {
  if (std::isnan(x)) return 0;
  double f = std::floor(x);
  double r = (x - f >= 0.5) ? f + 1.0 : f;
  if (r >= 9223372036854775807.0) return INT64_MAX;
  if (r <= -9223372036854775808.0) return INT64_MIN;
  return (int64_t)r;
}

// Java's double-to-int conversion (Scala Double.toInt): truncation toward
// zero, NaN gives 0, values beyond the int range saturate (JLS 5.1.3).
inline int32_t javaD2I(double x) {
  if (std::isnan(x)) return 0;
  if (x >= 2147483647.0) return INT32_MAX;
  if (x <= -2147483648.0) return INT32_MIN;
  return (int32_t)x;
}

// Scala Long.toInt: the low 32 bits.
inline int32_t javaL2I(int64_t x) { return (int32_t)(uint32_t)(uint64_t)x; }

inline int baseIndex(char c) {  // S/PileUp.scala:55-61
  switch (c) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    default: return -1;
  }
}
inline char indexBase(int i) { return "ACGT"[i]; }  // S/PileUp.scala:63

inline char upper(char c) { return (c >= 'a' && c <= 'z') ? (char)(c - 32) : c; }

// ---- BaseSum (S/BaseSum.scala:22-74) ---------------------------------------
// order: indices sorted by descending sum, stable (ties keep A<C<G<T).
inline void bsOrder(const int64_t s[4], int out[4]) {
  int idx[4] = {0, 1, 2, 3};
  std::stable_sort(idx, idx + 4, [&](int a, int b) { return s[a] > s[b]; });
  for (int i = 0; i < 4; i++) out[i] = idx[i];
}
inline int64_t bsSum(const int64_t s[4]) { return s[0] + s[1] + s[2] + s[3]; }
std::string bsToString(const int64_t s[4]) {
  return std::to_string(s[0]) + "," + std::to_string(s[1]) + "," + std::to_string(s[2]) + "," +
         std::to_string(s[3]);
}
std::string bsToStringPct(const int64_t s[4]) {
  int64_t div = bsSum(s);
  std::string o;
  for (int i = 0; i < 4; i++) {
    int64_t v = div == 0 ? 0 : (100 * s[i] + div / 2) / div;
    if (i) o += ",";
    o += std::to_string(v);
  }
  return o;
}

// ---- PileUp (S/PileUp.scala:25-267) ----------------------------------------
struct Params {
  int32_t minMq = 0, minQual = 0, flank = 10, defaultQual = 10, minMinDepth = 5;
  bool nonPf = false, duplicates = false, oldIndel = false, fixAmb = false;
  int32_t longRead = 0, bamType = 0;
  bool longReadOnly = false;
  double minDepth = 0.1;
};

struct PileUp {
  int64_t baseCount[4] = {0, 0, 0, 0};
  int64_t qualSum[4] = {0, 0, 0, 0};
  int32_t mqSum = 0, qSum = 0, physCov = 0, insertSize = 0, badPair = 0;
  int32_t deletions = 0, delQual = 0, insertions = 0, insQual = 0, clips = 0;
  std::vector<std::string> insertionList, deletionList;

  int64_t count() const { return bsSum(baseCount); }
  int64_t depth() const { return bsSum(baseCount) + deletions; }
  int64_t weightedMq() const { return roundDivL(bsSum(qualSum), qSum); }
  int64_t weightedQual() const { return roundDivL(bsSum(qualSum), mqSum); }
  int64_t meanQual() const { return roundDivL(bsSum(qualSum), roundDivL((int64_t)mqSum * count(), depth())); }
  int64_t meanMq() const { return roundDivL((int64_t)mqSum - depth(), depth()); }

  void add(char base, int32_t qual, int32_t mq, const Params& P) {  // :75-84
    int bi = baseIndex(base);
    if (bi >= 0 && qual >= P.minQual) {
      int32_t mq1 = mq + 1;
      baseCount[bi] += 1;
      qualSum[bi] += (int32_t)(qual * mq1);
      mqSum += mq1;
      qSum += qual;
    }
  }
  void addInsertion(const std::string& ins, int32_t qual, int32_t mq) {  // :97-104
    int32_t mq1 = mq + 1;
    insQual += mq1;
    qSum += qual;
    insertionList.push_back(ins);
    insertions += 1;
  }
  void addDeletion(const std::string& del, int32_t qual, int32_t mq) {  // :106-114
    int32_t mq1 = mq + 1;
    mqSum += mq1;
    delQual += mq1;
    qSum += qual;
    deletionList.push_back(del);
    deletions += 1;
  }
  int32_t insPct() const {  // :121
    return std::max(pctI(insQual, mqSum), pctI(insertions, (int32_t)count()));
  }
  int32_t delPct() const {  // :122
    return std::max(pctI(delQual, mqSum), pctI(deletions, (int32_t)count() + deletions));
  }
};

// PileUp.BaseCall (S/PileUp.scala:132-255)
struct BaseCall {
  int64_t n;
  int baseIdx, altIdx;
  char base, altBase;
  int64_t baseSum, altBaseSum;
  bool homo;
  int64_t score;
  std::string insertion, deletion;
  bool indel, homoIndel;

  bool isInsertion() const { return !insertion.empty(); }
  bool isDeletion() const { return !deletion.empty(); }
  bool called() const { return base != 'N' || indel; }
  int64_t q() const { return n > 0 ? score / n : 0; }
  bool highConfidence() const { return q() >= 10; }
  std::string callString(bool indelOk) const {
    if (indelOk && isInsertion()) return insertion;
    if (indelOk && isDeletion()) return deletion;
    return std::string(1, base);
  }
};

// hetIndelCall (S/PileUp.scala:209-247).  The winner must hold a strict
// majority, so the HashMap iteration order of the reference cannot matter.
static void hetIndelCall(const PileUp& pu, const std::vector<std::string>& list, int32_t pct,
                         const Params& P, std::string& call, bool& homo) {
  call.clear();
  homo = true;
  if (pu.depth() < P.minMinDepth || pct < 5 || list.empty()) return;
  std::map<std::string, int> counts;
  for (auto& s : list) counts[s] += 1;
  std::string win;
  int winCount = -1;
  for (auto& kv : counts)
    if (kv.second > winCount) { win = kv.first; winCount = kv.second; }
  if (winCount < 2 || winCount <= (int)list.size() / 2) return;
  if (win.find('N') != std::string::npos) return;
  int len = (int)win.size();
  if (P.oldIndel) {
    if (pct >= 33 && pct >= 50 - len) { call = win; homo = true; }
    return;
  }
  int middle = std::max(45 - len, 10);
  int low = middle / 2;
  int high = middle + middle - low;
  if (pct > high) { call = win; homo = true; }
  else if (pct >= low) { call = win; homo = false; }
}

BaseCall baseCall(const PileUp& pu, const Params& P) {
  BaseCall bc;
  bc.n = pu.count();
  int order[4];
  if (pu.qSum > 0) bsOrder(pu.qualSum, order); else bsOrder(pu.baseCount, order);
  bc.baseIdx = order[0];
  bc.altIdx = order[1];
  bc.base = bc.n > 0 ? indexBase(bc.baseIdx) : 'N';
  bc.baseSum = pu.qualSum[bc.baseIdx];
  bc.altBase = indexBase(bc.altIdx);
  bc.altBaseSum = pu.qualSum[bc.altIdx];
  {
    int64_t total = bsSum(pu.qualSum);
    int64_t homoScore = bc.baseSum - (total - bc.baseSum);
    int64_t halfTotal = total / 2;
    int64_t heteroScore = total - std::llabs(halfTotal - bc.baseSum) - std::llabs(halfTotal - bc.altBaseSum);
    bc.homo = homoScore >= heteroScore;
    bc.score = pu.mqSum > 0 ? std::llabs(homoScore - heteroScore) * bc.n / (int64_t)pu.mqSum : 0;
  }
  std::string ins, del;
  bool homoIns = true, homoDel = true;
  if (pu.insertions > 2 && pu.insertions > pu.deletions)
    hetIndelCall(pu, pu.insertionList, pu.insPct(), P, ins, homoIns);
  if (!ins.empty()) {
    bc.insertion = ins; bc.indel = true; bc.homoIndel = homoIns;
  } else {
    if (pu.deletions > 2 && pu.deletions > pu.insertions)
      hetIndelCall(pu, pu.deletionList, pu.delPct(), P, del, homoDel);
    if (!del.empty()) { bc.deletion = del; bc.indel = true; bc.homoIndel = homoDel; }
    else { bc.indel = false; bc.homoIndel = true; }
  }
  return bc;
}

// ---- Read view over the SoA feed --------------------------------------------
struct ReadView {
  const pg_reads* R;
  int64_t i;
  int32_t length() const { return R->l_seq[i]; }
  char base(int32_t k) const {
    if (k < 0 || k >= length()) throw IndexError();
    uint8_t b = R->seq[R->seq_off[i] + (k >> 1)];
    return kNib[(k & 1) ? (b & 15) : (b >> 4)];
  }
  std::string bases() const {
    std::string s((size_t)length(), ' ');
    for (int32_t k = 0; k < length(); k++) s[k] = base(k);
    return s;
  }
  bool hasQuals() const { return length() > 0 && R->qual[R->qual_off[i]] != 0xFF; }
  int32_t qual(int32_t k, const Params& P) const {
    if (k < 0 || k >= length()) throw IndexError();
    if (!hasQuals()) return (int32_t)(int8_t)P.defaultQual;
    return (int32_t)(int8_t)R->qual[R->qual_off[i] + k];
  }
  uint16_t flag() const { return R->flag[i]; }
  int32_t mq() const { return R->mapq[i]; }
};

inline bool consumesRead(int op) { return op == 0 || op == 1 || op == 4 || op == 7 || op == 8; }
inline bool consumesRef(int op) { return op == 0 || op == 2 || op == 3 || op == 7 || op == 8; }

// ---- PileUpRegion (S/PileUpRegion.scala:26-234) -------------------------------
struct PileUpRegion {
  int32_t start, stop;
  std::vector<PileUp> pileups;
  int64_t baseCount = 0;
  int32_t readCount = 0;
  int32_t physCovStart = 0, insertSizeStart = 0;
  const Params& P;

  PileUpRegion(int32_t s, int32_t e, const Params& p) : start(s), stop(e), pileups(e + 1 - s), P(p) {}
  int32_t size() const { return stop + 1 - start; }
  bool inRegion(int32_t l) const { return l >= start && l <= stop; }
  bool beforeRegion(int32_t l) const { return l < start; }
  int32_t index(int32_t l) const { return l - start; }
  int32_t locus(int32_t i) const { return start + i; }
  PileUp& at(int32_t idx) {
    if (idx < 0 || idx >= size()) throw IndexError();
    return pileups[idx];
  }
  int64_t coverage() const { return roundDivL(baseCount, size()); }

  void add(int32_t locus, char base, int32_t qual, int32_t mq, bool pair) {  // :38-48
    if (inRegion(locus)) {
      if (pair) {
        pileups[index(locus)].add(base, qual, mq, P);
        baseCount += 1;
      } else {
        pileups[index(locus)].badPair += 1;
      }
    }
  }
  void remove(int32_t locus, bool pair) {  // :50-58 (no-op for valid reads)
    if (inRegion(locus) && !pair) pileups[index(locus)].badPair -= 1;
  }

  int32_t physCovIncr(int32_t aStart, int32_t aEnd, int32_t iSize, bool paired, bool valid) {  // :62-88
    if (!valid || (paired && iSize <= 0)) return 0;
    int32_t s, e;
    if (!paired) { s = std::min(aStart, aEnd); e = std::max(aStart, aEnd); }
    else if (iSize > 0) { s = aStart; e = aStart + iSize; }
    else { s = aEnd + 1 + iSize; e = aEnd + 1; }
    int32_t insertSize = e - s;
    if (inRegion(s)) {
      pileups[index(s)].physCov += 1;
      pileups[index(s)].insertSize += insertSize;
    } else if (beforeRegion(s) && !beforeRegion(e)) {
      physCovStart += 1;
      insertSizeStart += insertSize;
    }
    if (inRegion(e)) {
      pileups[index(e)].physCov -= 1;
      pileups[index(e)].insertSize -= insertSize;
    }
    return insertSize;
  }

  void computePhysCov() {  // :90-100
    pileups[0].physCov += physCovStart;
    pileups[0].insertSize += insertSizeStart;
    for (int32_t i = 1; i < size(); i++) {
      pileups[i].physCov += pileups[i - 1].physCov;
      pileups[i].insertSize += pileups[i - 1].insertSize;
    }
    for (int32_t i = 0; i < size(); i++)
      if (pileups[i].physCov > 0) pileups[i].insertSize /= pileups[i].physCov;
  }

  int32_t addRead(const ReadView& r, const uint8_t* refBases, int64_t refLen, int32_t longRead) {  // :102-220
    const int32_t length = r.length();
    const int32_t mq = r.mq();
    const uint16_t fl = r.flag();
    const bool paired = fl & 0x1;
    const bool valid = (mq >= P.minMq) &&
                       ((!paired) || ((fl & 0x2) && r.R->ref_id[r.i] == r.R->mate_ref_id[r.i]));
    const int32_t insert = r.R->tlen[r.i];
    const int32_t aStart = r.R->pos[r.i];
    const int32_t aEnd = r.R->aend[r.i];
    int32_t readOffset = 0, refOffset = 0;
    const int32_t trustedFlank = P.flank;
    auto trusted = [&](int32_t off) { return off >= trustedFlank && length - trustedFlank > off; };
    auto ref = [&](int64_t k) -> uint8_t {
      if (k < 0 || k >= refLen) throw IndexError();
      return refBases[k];
    };
    auto homoRun = [&](int64_t i0) -> int64_t {  // :120-126
      uint8_t b = ref(i0);
      for (int64_t k = i0 + 1; k < refLen; k++)
        if (refBases[k] != b) return k - i0;
      return refLen - i0;
    };
    auto nanoporeExclude = [&](int64_t i0) -> bool {  // :128-134
      return inRegion(locus((int32_t)(i0 - 2))) && inRegion(locus((int32_t)(i0 + 2))) &&
             ref(i0 - 2) == 'C' && ref(i0 - 1) == 'C' && ref(i0 + 1) == 'G' && ref(i0 + 2) == 'G';
    };

    const int64_t co = r.R->cigar_off[r.i];
    const int nc = r.R->n_cigar[r.i];
    int32_t clippedBases = 0;  // :139
    for (int k = 0; k < nc; k++) {
      uint32_t w = r.R->cigar[co + k];
      if ((w & 15) == 4) clippedBases += (int32_t)(w >> 4);
    }
    const int32_t adjMq = roundDivI(mq * (length - clippedBases), length);  // :141
    const int32_t indelMq = longRead > 0 ? std::min(adjMq, 8) : adjMq;      // :142

    for (int k = 0; k < nc; k++) {  // :145-216
      uint32_t w = r.R->cigar[co + k];
      const int32_t len = (int32_t)(w >> 4);
      const int op = (int)(w & 15);
      const int32_t locus = aStart + refOffset;
      if (op == 1) {  // I
        int32_t iloc = locus;
        if (valid && trusted(readOffset) && inRegion(iloc)) {
          std::string insertion;  // bases.slice(readOffset, readOffset + len), clamped like slice
          for (int32_t j = std::max(readOffset, 0); j < std::min(readOffset + len, length); j++) insertion += r.base(j);
          while (iloc > 1) {
            uint8_t rb = ref(iloc - 2);
            if (len - 1 < 0 || len - 1 >= (int32_t)insertion.size()) throw IndexError();
            if (rb != (uint8_t)insertion[len - 1]) break;
            iloc -= 1;
            insertion = insertion.substr(len - 1, 1) + insertion.substr(0, len - 1);
          }
          if (!(longRead > 0 && homoRun(iloc) >= 4))
            at(index(iloc)).addInsertion(insertion, r.qual(readOffset, P), indelMq);
        }
      } else if (op == 2) {  // D
        int32_t dloc = locus;
        int32_t rloc = readOffset;
        if (valid && trusted(readOffset) && inRegion(dloc) && inRegion(dloc + len - 1)) {
          while (dloc > 1 && rloc > 0 && ref(dloc - 2) == ref((int64_t)dloc + len - 2)) {
            dloc -= 1;
            rloc -= 1;
            char base = r.base(rloc);
            int32_t qual = r.qual(rloc, P);
            if (trusted(rloc) && inRegion(dloc)) {
              remove(dloc, valid);
              if (inRegion(dloc + len)) add(dloc + len, base, qual, adjMq, valid);
            }
          }
          bool skip = false;
          if (longRead > 0) {
            skip = homoRun(index(dloc)) >= 4 || (longRead == PG_NANOPORE && nanoporeExclude(index(dloc)));
          }
          if (!skip) {
            std::string del;
            for (int64_t j = (int64_t)dloc - 1; j < (int64_t)dloc + len - 1; j++) {
              if (j >= 0 && j < refLen) del += (char)refBases[j];
            }
            at(index(dloc)).addDeletion(del, r.qual(readOffset, P), indelMq);
          }
        }
      } else if (op == 0 || op == 7 || op == 8) {  // M, =, X
        for (int32_t i = 0; i < len; i++) {
          int32_t rOff = readOffset + i;
          if (trusted(rOff)) {
            int32_t locusPlus = locus + i;
            char base = r.base(rOff);
            int32_t qual = (longRead == PG_NANOPORE && nanoporeExclude(index(locusPlus))) ? 0 : r.qual(rOff, P);
            add(locusPlus, base, qual, adjMq, valid);
          }
        }
      } else if (op == 4) {  // S
        int32_t clipStart = readOffset == 0 ? locus - len : locus;
        int32_t clipEnd = clipStart + len - 1;
        if (inRegion(clipStart)) pileups[index(clipStart)].clips += 1;
        if (inRegion(clipEnd)) pileups[index(clipEnd)].clips += 1;
        for (int32_t i = 0; i < len; i++) {
          int32_t rOff = readOffset + i;
          int32_t locusPlus = clipStart + i;
          (void)r.base(rOff);
          int32_t qual = r.qual(rOff, P);
          if (inRegion(locusPlus)) add(locusPlus, 'N', qual, adjMq, false);
        }
      }
      if (consumesRead(op)) readOffset += len;
      if (consumesRef(op)) refOffset += len;
    }
    readCount += 1;
    return physCovIncr(aStart, aEnd, insert, paired, valid);
  }
};

struct InsertStats {
  int64_t count = 0, sum = 0, sumSq = 0;
  void add(int32_t size) {  // S/BamFile.scala:161-165
    sum += size;
    sumSq += (int32_t)(size * size);
    count += 1;
  }
};

// S/BamFile.scala:101-105
bool validateRead(uint16_t fl, const Params& P) {
  return (P.nonPf || !(fl & 0x200)) && (P.duplicates || !(fl & 0x400)) && !(fl & 0x100);
}

int32_t hugeInsert(int32_t bamType) {  // S/BamFile.scala:29, 192
  int32_t m = bamType == PG_BAM_FRAGS ? 500 : 10000;
  return 5 * m;
}

// ---- GenomeRegion (S/GenomeRegion.scala) ------------------------------------
enum ChangeKind { SNP = 1, INS = 2, DEL = 3, AMB = 4 };

struct Fix {
  int32_t locus;
  std::string was, patch;
  int src;  // 0 snp, 1 small, 2 big
  bool operator==(const Fix& o) const { return locus == o.locus && was == o.was && patch == o.patch; }
};

struct GenomeRegion;
// Local reassembly of one gap or break (GapFiller.fillGap / fixBreak,
// S/GapFiller.scala:39-100) with the BAM's insert statistics as the region
// sees them; defined with the graph walk below.
struct Reassembly;
struct BamStats;
Fix reassemble(const GenomeRegion& g, const Reassembly& ra, const BamStats& st, int32_t bs, int32_t be, bool isGap,
               int64_t& tiedSets);

struct GenomeRegion {
  std::string name;
  int32_t contigId;
  const uint8_t* contigBases;
  int64_t contigLen;
  int32_t start, stop;
  const Params& P;
  PileUpRegion pr;
  std::vector<uint8_t> bases;  // current (fixed) bases
  std::vector<uint8_t> confirmed, ambiguous, changed, deleted, excluded;
  std::vector<int32_t> coverage, badCoverage, clips, physCoverage, insertSizeA, fragCoverage;
  std::vector<int16_t> copyNumber;
  std::map<int32_t, std::pair<int, int32_t>> changeMap;  // index -> (kind, index)
  int32_t minDepth;
  InsertStats fr, rf;
  std::vector<Fix> snpFixList, smallFixList, bigFixList;  // prepend order kept by building reversed

  GenomeRegion(const std::string& nm, int32_t cid, const uint8_t* cb, int64_t clen, int32_t s, int32_t e,
               const Params& p)
      : name(nm), contigId(cid), contigBases(cb), contigLen(clen), start(s), stop(e), P(p), pr(s, e, p) {
    int32_t n = size();
    bases.assign(cb + (s - 1), cb + e);
    confirmed.assign(n, 0); ambiguous.assign(n, 0); changed.assign(n, 0);
    deleted.assign(n, 0); excluded.assign(n, 0);
    coverage.assign(n, 0); badCoverage.assign(n, 0); clips.assign(n, 0);
    physCoverage.assign(n, 0); insertSizeA.assign(n, 0); fragCoverage.assign(n, 0);
    copyNumber.assign(n, 0);
    minDepth = p.minMinDepth;
  }
  int32_t size() const { return stop + 1 - start; }
  bool inRegion(int32_t l) const { return l >= start && l <= stop; }
  int32_t index(int32_t l) const { return l - start; }
  int32_t locus(int32_t i) const { return start + i; }
  char refBase(int32_t l) const {  // :783-787
    if (!inRegion(l)) throw IndexError();
    return upper((char)contigBases[l - 1]);
  }
  char baseAt(int32_t l) const {  // :766-769 (bases = original during postProcess)
    if (!inRegion(l)) throw IndexError();
    return upper((char)bases[index(l)]);
  }

  // BamFile.process (S/BamFile.scala:108-148) + processBam (:287-300)
  void processBam(const pg_reads* R, int64_t rb, int64_t re) {
    std::vector<int32_t> covBefore(size());
    bool jumps = P.bamType == PG_BAM_JUMPS;
    if (!jumps)
      for (int32_t i = 0; i < size(); i++) covBefore[i] = (int32_t)pr.pileups[i].depth();
    int64_t qs = std::max<int64_t>((int64_t)start - 10000, 0);
    int64_t qe = std::min<int64_t>((int64_t)stop + 10000, contigLen);
    int32_t huge = hugeInsert(P.bamType);
    for (int64_t i = rb; i < re; i++) {
      if (R->ref_id[i] != contigId) continue;
      int64_t rs = R->pos[i];
      int64_t rend = (R->flag[i] & 0x4) ? R->pos[i] : R->aend[i];
      if (!(rs <= qe && rend >= qs)) continue;
      if (!validateRead(R->flag[i], P)) continue;
      ReadView rv{R, i};
      int32_t insertSize = pr.addRead(rv, contigBases, contigLen, P.longRead);
      bool rc = R->flag[i] & 0x10;
      bool frr = (insertSize > 0) ^ rc;
      if (insertSize > 0 && insertSize < huge) {
        if (frr) fr.add(insertSize); else rf.add(insertSize);
      }
    }
    if (!jumps)
      for (int32_t i = 0; i < size(); i++) fragCoverage[i] += (int32_t)pr.pileups[i].depth() - covBefore[i];
  }

  int32_t homoRunG(int32_t loc) const {  // :416-422
    char b = baseAt(loc);
    for (int32_t i = loc; i <= stop; i++)
      if (baseAt(i) != b) return i - loc;
    return 1 + stop - loc;
  }
  bool nanoporeExcludeG(int32_t loc) const {  // :424-430
    return inRegion(loc - 2) && inRegion(loc + 2) && baseAt(loc - 2) == 'C' && baseAt(loc - 1) == 'C' &&
           baseAt(loc + 1) == 'G' && baseAt(loc + 2) == 'G';
  }

  static std::vector<int32_t> smooth(const std::vector<int32_t>& input, int32_t window) {  // :190-210
    int32_t inputSize = (int32_t)input.size();
    std::vector<int32_t> result(inputSize, 0);
    int32_t half = window / 2;
    int32_t accum = 0;
    for (int32_t i = 0; i < inputSize; i++) {
      accum += input[i];
      if (i > window) {
        accum -= input[i - window];
        result[i - half] = (accum + half) / window;
      }
    }
    if (inputSize > window) {
      for (int32_t i = 0; i < window - half; i++) result[i] = result[window - half];
      for (int32_t i = inputSize - half; i < inputSize; i++) result[i] = result[inputSize - half - 1];
    } else {
      for (int32_t i = 0; i < inputSize; i++) result[i] = accum / inputSize;
    }
    return result;
  }
  double fragMean() const {  // NormalDistribution.mean (S/NormalDistribution.scala:29)
    double s = 0;
    for (int32_t v : fragCoverage) s += (double)v;
    return s / (double)fragCoverage.size();
  }

  void postProcess() {  // :214-285
    pr.computePhysCov();
    int64_t meanCoverage = pr.coverage();
    int32_t nReads = pr.readCount;
    if (P.longReadOnly) {  // excludeMotifs (:432-439)
      bool nano = P.longRead == PG_NANOPORE;
      for (int32_t i = 0; i < size(); i++)
        excluded[i] = homoRunG(locus(i)) >= 4 || (nano && nanoporeExcludeG(locus(i)));
    }
    if (P.minDepth >= 1) minDepth = javaD2I(P.minDepth);
    else minDepth = std::max(javaL2I(javaRound(P.minDepth * (double)meanCoverage)), P.minMinDepth);
    if (nReads == 0) return;
    bool fixamb = P.fixAmb;
    for (int32_t i = 0; i < size(); i++) {
      PileUp& pu = pr.pileups[i];
      int64_t n = pu.depth();
      BaseCall bc = baseCall(pu, P);
      char b = bc.base;
      bool homo = bc.homo;
      char r = refBase(i + start);
      coverage[i] = (int32_t)n;
      badCoverage[i] = pu.badPair;
      physCoverage[i] = pu.physCov;
      insertSizeA[i] = pu.insertSize;
      clips[i] = (int16_t)pu.clips;
      if (n >= minDepth && r != 'N' && !deleted[i] && bc.called()) {
        if (homo && b == r && bc.highConfidence() && !bc.indel) confirmed[i] = 1;
        else if (bc.isInsertion() && bc.homoIndel) addChange(i, INS);
        else if (bc.isDeletion() && bc.homoIndel) {
          addChange(i, DEL);
          for (int32_t j = 1; j < (int32_t)bc.deletion.size(); j++) {
            if (i + j >= size()) throw IndexError();
            deleted[i + j] = 1;
            pr.pileups[i + j].deletions += pu.deletions;
          }
        } else if (b != r && bc.score > 0) {
          if (homo) addChange(i, SNP);
          else if (fixamb || bc.altBase != r) addChange(i, AMB);
        }
      }
    }
    double baseCov = fragMean();
    std::vector<int32_t> smoothCov = smooth(fragCoverage, 200);
    for (int32_t i = 0; i < size(); i++) {
      int32_t nn = smoothCov[i];
      copyNumber[i] = baseCov > 0 ? (int16_t)javaRound((double)nn / baseCov) : (int16_t)0;
    }
  }
  void addChange(int32_t i, int kind) {  // :85-89
    if (kind == AMB) ambiguous[i] = 1; else changed[i] = 1;
    changeMap[i] = {kind, i};
  }

  int64_t tiedSets = 0;  // see breakJoins in reassemble

  // identifyAndFixIssues (:307-414); ra and st (fix types gaps / local) may be null
  void identifyAndFixIssues(bool fixSnps, bool fixIndels, bool iupac, bool longread, const Reassembly* ra = nullptr,
                            const BamStats* st = nullptr, bool fixGaps = false, bool fixLocal = false) {
    for (auto& kv : changeMap) {
      int32_t i = kv.first;
      int kind = kv.second.first;
      int32_t loc = locus(i);
      char rBase = refBase(loc);
      BaseCall bc = baseCall(pr.pileups[i], P);
      char cBase = bc.base;
      if (!excluded[i]) {
        if (kind == SNP) {
          if (fixSnps) snpFixList.push_back({loc, std::string(1, rBase), std::string(1, cBase), 0});
        } else if (kind == AMB) {
          if (fixSnps && !longread) {
            if (iupac) smallFixList.push_back({loc, std::string(1, rBase), std::string(1, toIUPAC(cBase, bc.altBase)), 1});
            else snpFixList.push_back({loc, std::string(1, rBase), std::string(1, cBase), 0});
          }
        } else if (kind == INS) {
          if (fixIndels) smallFixList.push_back({loc, "", bc.insertion, 1});
        } else if (kind == DEL) {
          if (fixIndels) smallFixList.push_back({loc, bc.deletion, "", 1});
        }
      }
    }
    // The reference prepends (::=), so its lists run in descending locus order.
    std::reverse(snpFixList.begin(), snpFixList.end());
    std::reverse(smallFixList.begin(), smallFixList.end());
    fixIssues(snpFixList);
    if (ra && fixGaps) {  // :383-393, each gap in locus order
      for (auto& gp : gaps()) {
        Fix f = reassemble(*this, *ra, *st, gp.first, gp.second, true, tiedSets);
        if (f.locus > 0) bigFixList.push_back(f);
      }
    }
    if (ra && fixLocal) {  // :396-410
      for (auto& br : possibleBreaks()) {
        Fix f = reassemble(*this, *ra, *st, br.first, br.second, false, tiedSets);
        if (f.locus > 0 && std::max(f.was.size(), f.patch.size()) > 10) bigFixList.push_back(f);
      }
    }
    std::reverse(bigFixList.begin(), bigFixList.end());  // prepended (::=) in the reference
    std::vector<Fix> sb = smallFixList;
    sb.insert(sb.end(), bigFixList.begin(), bigFixList.end());
    fixIssues(sb);
  }
  static char toIUPAC(char a, char b) {  // S/Bases.scala:85-88
    int bits = (1 << baseIndex(a)) | (1 << baseIndex(b));
    switch (bits) {
      case 1: return 'A'; case 2: return 'C'; case 4: return 'G'; case 8: return 'T';
      case 5: return 'R'; case 10: return 'Y'; case 6: return 'S'; case 9: return 'W';
      case 12: return 'K'; case 3: return 'M'; case 14: return 'B'; case 13: return 'D';
      case 11: return 'H'; case 7: return 'V'; case 15: return 'N';
    }
    return 'N';
  }

  std::vector<Fix> fixFixList(const std::vector<Fix>& inList) const {  // :557-593
    std::vector<Fix> fixes = inList;
    std::stable_sort(fixes.begin(), fixes.end(), [](const Fix& x, const Fix& y) { return x.locus < y.locus; });
    std::vector<Fix> out;
    size_t h = 0;  // fixes[h..] is the working list; fixes[h] may be replaced
    while (h < fixes.size()) {
      if (h + 1 < fixes.size()) {
        const Fix& f1 = fixes[h];
        const Fix& f2 = fixes[h + 1];
        int32_t s1 = f1.locus, e1 = f1.locus + std::max((int32_t)f1.was.size() - 1, 0);
        int32_t s2 = f2.locus, e2 = f2.locus + std::max((int32_t)f2.was.size() - 1, 0);
        bool overlaps = s2 <= e1 && e2 >= s1;
        if (overlaps) {
          size_t l1 = f1.was.size() + f1.patch.size(), l2 = f2.was.size() + f2.patch.size();
          if (l1 >= l2) fixes[h + 1] = f1;
          h += 1;
        } else {
          out.push_back(f1);
          h += 1;
        }
      } else {
        out.push_back(fixes[h]);
        h += 1;
      }
    }
    return out;
  }

  void fixIssues(const std::vector<Fix>& fixList) {  // :595-621
    std::vector<uint8_t> newBases = bases;
    std::vector<Fix> fl = fixFixList(fixList);
    for (auto it = fl.rbegin(); it != fl.rend(); ++it) {
      const Fix& f = *it;
      int32_t s = index(f.locus);
      if (f.was.size() == f.patch.size()) {
        for (size_t i = 0; i < f.was.size(); i++) newBases[s + i] = (uint8_t)f.patch[i];
      } else {
        std::vector<uint8_t> nb(newBases.begin(), newBases.begin() + s);
        nb.insert(nb.end(), f.patch.begin(), f.patch.end());
        size_t a = std::min(newBases.size(), (size_t)s + f.was.size());
        nb.insert(nb.end(), newBases.begin() + a, newBases.end());
        newBases.swap(nb);
      }
    }
    bases = newBases;
  }

  std::vector<Fix> allFixes() const {
    std::vector<Fix> all = snpFixList;
    all.insert(all.end(), smallFixList.begin(), smallFixList.end());
    all.insert(all.end(), bigFixList.begin(), bigFixList.end());
    return fixFixList(all);
  }

  // summaryRegions (:743-763); returns [first,last] loci pairs
  template <class F>
  std::vector<std::pair<int32_t, int32_t>> summaryRegions(F test, int32_t slop = 100) const {
    std::vector<std::pair<int32_t, int32_t>> regs;
    int32_t first = -1, last = -1;
    for (int32_t i = 0; i < size(); i++) {
      if (test(i)) {
        last = i;
        if (first < 0) first = i;
      } else if (last >= 0 && i > last + slop) {
        regs.push_back({locus(first), locus(last)});
        first = -1;
        last = -1;
      }
    }
    if (last >= 0) regs.push_back({locus(first), locus(last)});
    std::vector<std::pair<int32_t, int32_t>> out;
    for (auto& r : regs)
      if (!(r.first - start < 100 || stop - r.second < 100)) out.push_back(r);  // nearEdge
    return out;
  }
  std::vector<std::pair<int32_t, int32_t>> duplicationEvents() const {  // :735-741
    auto regs = summaryRegions([&](int32_t i) { return copyNumber[i] > 1; }, 2000);
    std::vector<std::pair<int32_t, int32_t>> out;
    for (auto& r : regs)
      if (r.second + 1 - r.first > 10000) out.push_back(r);
    return out;
  }
  int64_t pctBadOverall() const {  // :99-114
    int64_t bad = 0, good = 0;
    for (int32_t i = 0; i < size(); i++) { bad += badCoverage[i]; good += coverage[i]; }
    return pctL(bad, good + bad);
  }
  std::vector<std::pair<int32_t, int32_t>> gaps() const {  // :700
    auto gapsR = summaryRegions([&](int32_t i) { return refBase(locus(i)) == 'N'; });
    std::vector<std::pair<int32_t, int32_t>> out;
    for (auto& g : gapsR)
      if (g.second + 1 - g.first >= 10) out.push_back(g);
    return out;
  }
  // :771-781: originalBaseAt, subString (current bases), refSubString (the contig)
  char originalBaseAt(int32_t l) const {
    if (!inRegion(l)) throw IndexError();
    return upper((char)contigBases[l - 1]);
  }
  std::string subString(int32_t l, int32_t n) const {
    if (!(inRegion(l) && inRegion(l + n - 1))) throw IndexError();
    std::string s;
    for (int32_t k = index(l); k < index(l + n); k++) s.push_back(upper((char)bases[k]));
    return s;
  }
  std::string refSubString(int32_t l, int32_t n) const {
    if (!(inRegion(l) && inRegion(l + n - 1))) throw IndexError();
    std::string s;
    for (int32_t k = l - 1; k < l + n - 1; k++) s.push_back(upper((char)contigBases[k]));
    return s;
  }
  std::vector<std::pair<int32_t, int32_t>> possibleBreaks() const {  // :659-720
    double mean = fragMean();
    int64_t pbo = pctBadOverall();
    auto gaps = this->gaps();
    auto breakp = [&](int32_t i) {
      bool lowCov = coverage[i] < P.minMinDepth && refBase(locus(i)) != 'N';
      bool highClip = coverage[i] >= P.minMinDepth && pctI(clips[i], coverage[i]) >= 33;
      int32_t good = coverage[i], bad = badCoverage[i];
      bool tooBad = pctI(bad, good + bad) > pbo + 20;
      int32_t left = fragCoverage[std::max(0, i - 100)];
      int32_t right = fragCoverage[std::min(size() - 1, i + 100)];
      int32_t center = fragCoverage[i];
      double dipF = (double)((left - center) + (right - center)) / mean;
      return lowCov || highClip || tooBad || dipF >= 1.5;
    };
    auto regs = summaryRegions(breakp, 200);
    std::vector<std::pair<int32_t, int32_t>> out;
    for (auto& r : regs) {
      bool near = false;
      for (auto& g : gaps) {  // Region.near (S/Region.scala:41-43), distance 300
        bool ov = g.first <= r.second && g.second >= r.first;
        if (ov || std::abs(g.second - r.first) <= 300 || std::abs(g.first - r.second) <= 300) near = true;
      }
      if (!near) out.push_back(r);
    }
    return out;
  }
};

// ---- VCF (S/Vcf.scala) --------------------------------------------------------
// Java's "%.2f" on a double: shortest round-trip decimal digits, then HALF_UP.
std::string javaFormat2(double x) {
  char buf[64];
  auto res = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::fixed);
  std::string s(buf, res.ptr);
  bool neg = false;
  if (!s.empty() && s[0] == '-') { neg = true; s = s.substr(1); }
  size_t dot = s.find('.');
  std::string ip = dot == std::string::npos ? s : s.substr(0, dot);
  std::string fp = dot == std::string::npos ? "" : s.substr(dot + 1);
  while (fp.size() < 3) fp += '0';
  std::string digits = ip + fp.substr(0, 2);
  bool up = fp[2] >= '5';
  if (up) {
    int k = (int)digits.size() - 1;
    while (k >= 0) {
      if (digits[k] == '9') { digits[k] = '0'; k--; }
      else { digits[k] += 1; break; }
    }
    if (k < 0) digits = "1" + digits;
  }
  std::string out = digits.substr(0, digits.size() - 2) + "." + digits.substr(digits.size() - 2);
  return (neg ? "-" : "") + out;
}

struct VcfWriter {
  FILE* f;
  bool diploid = false, vcfQE = false;
  const Params& P;
  void header(const std::vector<std::pair<std::string, int64_t>>& contigs, const char* date, const char* source,
              const char* args, const char* ref) {  // :28-68
    fprintf(f, "##fileformat=VCFv4.1\n##fileDate=%s\n##source=\"%s\"\n##PILON=\"%s\"\n##reference=%s\n", date,
            source, args, ref);
    for (auto& c : contigs) fprintf(f, "##contig=<ID=%s,length=%lld>\n", c.first.c_str(), (long long)c.second);
    fputs("##FILTER=<ID=LowCov,Description=\"Low Coverage of good reads at location\">\n"
          "##FILTER=<ID=Amb,Description=\"Ambiguous evidence in haploid genome\">\n"
          "##FILTER=<ID=Del,Description=\"This base is in a deletion or change event from another record\">\n"
          "##INFO=<ID=DP,Number=1,Type=Integer,Description=\"Valid read depth; some reads may have been filtered\">\n"
          "##INFO=<ID=TD,Number=1,Type=Integer,Description=\"Total read depth including bad pairs\">\n"
          "##INFO=<ID=PC,Number=1,Type=Integer,Description=\"Physical coverage of valid inserts across locus\">\n"
          "##INFO=<ID=BQ,Number=1,Type=Integer,Description=\"Mean base quality at locus\">\n"
          "##INFO=<ID=MQ,Number=1,Type=Integer,Description=\"Mean read mapping quality at locus\">\n"
          "##INFO=<ID=QD,Number=1,Type=Integer,Description=\"Variant confidence/quality by depth\">\n"
          "##INFO=<ID=BC,Number=4,Type=Integer,Description=\"Count of As, Cs, Gs, Ts at locus\">\n",
          f);
    if (vcfQE)
      fputs("##INFO=<ID=QE,Number=4,Type=Integer,Description=\"Evidence for As, Cs, Gs, Ts weighted by Q & MQ at locus\">\n", f);
    else
      fputs("##INFO=<ID=QP,Number=4,Type=Integer,Description=\"Percentage of As, Cs, Gs, Ts weighted by Q & MQ at locus\">\n", f);
    fputs("##INFO=<ID=IC,Number=1,Type=Integer,Description=\"Number of reads with insertion here\">\n"
          "##INFO=<ID=DC,Number=1,Type=Integer,Description=\"Number of reads with deletion here\">\n"
          "##INFO=<ID=XC,Number=1,Type=Integer,Description=\"Number of reads clipped here\">\n"
          "##INFO=<ID=AC,Number=A,Type=Integer,Description=\"Allele count in genotypes, for each ALT allele, in the same order as listed\">\n"
          "##INFO=<ID=AF,Number=A,Type=Float,Description=\"Fraction of evidence in support of alternate allele(s)\">\n"
          "##INFO=<ID=SVTYPE,Number=1,Type=String,Description=\"Type of structural variant\">\n"
          "##INFO=<ID=SVLEN,Number=.,Type=String,Description=\"Difference in length between REF and ALT alleles\">\n"
          "##INFO=<ID=END,Number=1,Type=Integer,Description=\"End position of the variant described in this record\">\n"
          "##INFO=<ID=IMPRECISE,Number=0,Type=Flag,Description=\"Imprecise change from local reassembly (ALT contains Ns)\">\n"
          "##FORMAT=<ID=GT,Number=1,Type=String,Description=\"Genotype\">\n"
          "##FORMAT=<ID=AD,Number=.,Type=String,Description=\"Allelic depths for the ref and alt alleles in the order listed\">\n"
          "##FORMAT=<ID=DP,Number=1,Type=String,Description=\"Approximate read depth; some reads may have been filtered\">\n"
          "##ALT=<ID=DUP,Description=\"Possible segmental duplication\">\n"
          "#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT\tSAMPLE\n",
          f);
  }

  void writeRecord(GenomeRegion& g, int32_t index, bool embedded, bool indelOkArg) {  // :74-176
    bool indelOk = indelOkArg && index > 0;
    int32_t locus = g.locus(index);
    const PileUp& pu = g.pr.pileups[index];
    BaseCall bc = baseCall(pu, P);
    std::string bcString = bc.callString(indelOk);
    int32_t baseDP = (int32_t)bc.baseSum;
    int32_t altBaseDP = (int32_t)bc.altBaseSum;
    int32_t depth = (int32_t)pu.depth();
    int32_t loc = locus;
    std::string rBase, cBase, callType;
    int32_t refDP, altDP;
    if (indelOk && !embedded && bc.isDeletion()) {
      loc -= 1;
      char rb = g.refBase(loc);
      callType = bc.homoIndel ? "1/1" : "0/1";
      int32_t p = pu.delPct();
      rBase = std::string(1, rb) + bcString; cBase = std::string(1, rb); refDP = 100 - p; altDP = p;
    } else if (indelOk && !embedded && bc.isInsertion()) {
      loc -= 1;
      char rb = g.refBase(loc);
      callType = bc.homoIndel ? "1/1" : "0/1";
      int32_t p = pu.insPct();
      rBase = std::string(1, rb); cBase = std::string(1, rb) + bcString; refDP = 100 - p; altDP = p;
    } else if (bc.homo) {
      char rb = g.refBase(loc);
      rBase = std::string(1, rb);
      if (rb == bc.base || bcString == "N") { cBase = std::string(1, bc.base); callType = "0/0"; refDP = baseDP; altDP = altBaseDP; }
      else { cBase = std::string(1, bc.base); callType = "1/1"; refDP = altBaseDP; altDP = baseDP; }
    } else {
      char rb = g.refBase(loc);
      rBase = std::string(1, rb);
      if (rb == bc.base) { cBase = std::string(1, bc.altBase); callType = "0/1"; refDP = baseDP; altDP = altBaseDP; }
      else { cBase = std::string(1, bc.base); callType = "0/1"; refDP = altBaseDP; altDP = baseDP; }
    }
    std::vector<std::string> filters;  // prepended in the reference; built reversed here
    if (depth < g.minDepth) filters.insert(filters.begin(), "LowCov");
    if (!diploid && callType == "0/1") filters.insert(filters.begin(), "Amb");
    if (embedded) filters.insert(filters.begin(), "Del");
    if (filters.empty()) filters.push_back("PASS");
    std::string cBaseVcf = (cBase == "N" || cBase == rBase) ? "." : cBase;
    std::string filter;
    for (size_t k = 0; k < filters.size(); k++) { if (k) filter += ";"; filter += filters[k]; }
    int ac = callType == "0/0" ? 0 : callType == "0/1" ? 1 : 2;
    double af = 0.0;
    int32_t tot = refDP + altDP;
    if (tot > 0 && cBaseVcf != ".") af = (double)((float)altDP / (float)tot);
    std::string info = "DP=" + std::to_string(!embedded ? pu.depth() : pu.count()) +
                       ";TD=" + std::to_string(pu.depth() + pu.badPair) +
                       ";BQ=" + std::to_string(pu.meanQual()) + ";MQ=" + std::to_string(pu.meanMq()) +
                       ";QD=" + std::to_string(bc.q()) + ";BC=" + bsToString(pu.baseCount) +
                       (vcfQE ? ";QE=" + bsToString(pu.qualSum) : ";QP=" + bsToStringPct(pu.qualSum)) +
                       ";PC=" + std::to_string(pu.physCov) + ";IC=" + std::to_string(pu.insertions) +
                       ";DC=" + std::to_string(pu.deletions) + ";XC=" + std::to_string(pu.clips) +
                       ";AC=" + std::to_string(ac) + ";AF=" + javaFormat2(af);
    std::string qual = (indelOk && bc.isDeletion()) ? "." : std::to_string(bc.score);
    fprintf(f, "%s\t%d\t.\t%s\t%s\t%s\t%s\t%s\tGT\t%s\n", g.name.c_str(), loc, rBase.c_str(), cBaseVcf.c_str(),
            qual.c_str(), filter.c_str(), info.c_str(), callType.c_str());
    if (indelOk && bc.indel && !embedded) writeRecord(g, index, bc.isDeletion() && bc.homoIndel, false);
  }

  void writeDup(GenomeRegion& g, std::pair<int32_t, int32_t> d) {  // :194-202
    int32_t loc = d.first - 1;
    char rb = g.refBase(loc);
    fprintf(f, "%s\t%d\t.\t%c\t<DUP>\t.\tPASS\tSVTYPE=DUP;SVLEN=%d;END=%d;IMPRECISE\tGT\t./.\n", g.name.c_str(), loc,
            rb, d.second + 1 - d.first, d.second);
  }

  void writeFixRecord(GenomeRegion& g, const Fix& fx) {  // :178-192
    int32_t loc = fx.locus - 1;
    char rb = g.refBase(loc);
    std::string ref = std::string(1, rb) + fx.was, alt = std::string(1, rb) + fx.patch;
    int32_t svlen = (int32_t)alt.size() - (int32_t)ref.size();
    int32_t svend = loc + (int32_t)ref.size() - 1;
    fprintf(f, "%s\t%d\t.\t%s\t%s\t.\tPASS\tSVTYPE=%s;SVLEN=%d;END=%d%s\tGT\t1/1\n", g.name.c_str(), loc, ref.c_str(),
            alt.c_str(), svlen < 0 ? "DEL" : "INS", svlen, svend,
            fx.patch.find('N') != std::string::npos ? ";IMPRECISE" : "");
  }

  void writeRegion(GenomeRegion& g) {  // GenomeRegion.writeVcf (:623-643)
    std::vector<Fix> fixes = g.allFixes();
    auto dupes = g.duplicationEvents();
    auto in = [](const std::vector<Fix>& l, const Fix& x) { return std::find(l.begin(), l.end(), x) != l.end(); };
    size_t fh = 0, dh = 0;
    for (int32_t i = 0; i < g.size(); i++) {
      int32_t loc = g.locus(i);
      if (dh < dupes.size() && dupes[dh].first == loc) { writeDup(g, dupes[dh]); dh++; }
      if (fh < fixes.size() && fixes[fh].locus == loc) {
        const Fix& fx = fixes[fh];
        if (in(g.bigFixList, fx) && !in(g.smallFixList, fx)) {  // a local reassembly
          writeFixRecord(g, fx);
          for (size_t j = 0; j < fx.was.size(); j++) {
            if (i + (int32_t)j >= g.size()) throw IndexError();
            g.deleted[i + j] = 1;
          }
        }
        fh++;
      }
      writeRecord(g, i, g.deleted[i] != 0, true);
    }
  }
};

// ---- Local reassembly ---------------------------------------------------------
// BamFile.scan / MateMap / recruitment (S/BamFile.scala:156-220, 222-403), the
// Assembler's K-mer tally and graph walk (S/Assembler.scala:46-284) and the
// GapFiller (S/GapFiller.scala:28-402) for one BAM of type frags or unpaired.
// Read names are given as ids (mates share an id); Pilon.trSafe is always
// true and Pilon.multiClosure / fixNovel are off (their defaults).

static double isMean(const InsertStats& s) {  // :167
  return s.count > 0 ? (double)s.sum / (double)s.count : 0.0;
}
static double isSigma(const InsertStats& s) {  // :169-173
  if (s.sum > 0) return std::sqrt(std::fabs((double)s.sumSq / (double)s.count - isMean(s) * isMean(s)));
  return 0.0;
}
static int32_t isMaxInsert(const InsertStats& s) {  // :181-183
  return s.count > 1000 ? javaL2I(javaRound(isMean(s) + 3.0 * isSigma(s))) : 0;
}

static std::string revComp(const std::string& s) {  // S/Bases.scala:28-40
  std::string r(s.rbegin(), s.rend());
  for (auto& c : r) c = c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : c == 'T' ? 'A' : c;
  return r;
}

// Assembler.addReads + buildGraph (S/Assembler.scala:46-87, 132-154) over reads
// `idx` in that order; returns the K-mer -> pileup map before the depth filter.
static std::unordered_map<std::string, PileUp> tallyReads(const pg_reads* R, const Params& P, const int64_t* idx,
                                                          int64_t n, int32_t K) {
  std::unordered_map<std::string, PileUp> pileups;
  int64_t nReads = 0;
  auto addToPileups = [&](const std::string& b, const std::vector<int32_t>& q, int32_t mq) {
    int32_t length = (int32_t)b.size();
    for (int32_t off = 0; off <= length - K - 1; off++) {
      PileUp& pu = pileups[b.substr(off, K)];
      pu.add(b[off + K], q[off + K], mq, P);
    }
  };
  for (int64_t t = 0; t < n; t++) {
    ReadView rv{R, idx[t]};
    std::string b = rv.length() > 0 ? rv.bases() : std::string("*");
    int32_t length = (int32_t)b.size();
    if (length > K) {
      std::vector<int32_t> q(length);
      for (int32_t k = 0; k < length; k++) q[k] = rv.qual(k, P);
      int32_t mq = rv.mq();
      addToPileups(b, q, mq);
      std::vector<int32_t> rq(q.rbegin(), q.rend());
      addToPileups(revComp(b), rq, mq);
      nReads++;
      if (nReads % 100000 == 0) {  // prunePileups(2)
        for (auto it = pileups.begin(); it != pileups.end();)
          if (it->second.count() < 2) it = pileups.erase(it); else ++it;
      }
    }
  }
  return pileups;
}

// BamFile's insert statistics (S/BamFile.scala:156-220): insertStatsFR / RF /
// Unpaired, and what GapFiller reads of them.
struct BamStats {
  InsertStats fr, rf, un;
  int32_t bamType = PG_BAM_FRAGS;
  void addInsert(int32_t insertSize, bool rc, bool unpaired) {  // :194-202
    bool frr = (insertSize > 0) ^ rc;
    if (insertSize > 0 && insertSize < hugeInsert(bamType)) {
      if (unpaired) un.add(insertSize); else if (frr) fr.add(insertSize); else rf.add(insertSize);
    }
  }
  void addRegion(const GenomeRegion& g);  // BamFile.process's addInsert calls (:137)
  int64_t pctFR() const { return pctL(fr.count, fr.count + rf.count + un.count); }  // :204
  double insertSizeMean() const { return pctFR() >= 50 ? isMean(fr) : isMean(rf); }  // :208-210
  int32_t maxInsertSize() const {  // :216-220
    int32_t m = std::max(isMaxInsert(fr), std::max(isMaxInsert(rf), isMaxInsert(un)));
    return m > 0 ? m : (bamType == PG_BAM_FRAGS ? 500 : 10000);
  }
  int32_t breakRadius(int32_t K) const {  // S/GapFiller.scala:357-362 (one frags BAM, or none)
    int32_t insertMean = bamType == PG_BAM_FRAGS ? javaL2I(javaRound(insertSizeMean())) : 0;
    return std::max(3 * K, insertMean);
  }
};

struct Reassembly {
  const pg_reads* R;
  const int64_t* nameId;  // the read name of each read as an id; null: no names (no stray mates)
  const Params& P;
  int32_t K;
  bool strays;
  bool fixBreaks = false;  // --fix breaks (--variant): breaks get the partial fill of gaps
  int32_t gapMargin = 100000;  // Pilon.gapMargin (--gapmargin)
  int32_t minGap = 10;         // Pilon.minGap (--mingap)
  BamStats scanStats;      // the statistics of BamFile.scan
  std::unordered_map<int64_t, int64_t> stray1, stray2;  // strayMateMap readMap1 / readMap2 (:222-281)
  std::vector<int64_t> cb, ce;                           // each contig's read range
  std::vector<int32_t> span;                             // longest alignment span of each contig's reads

  Reassembly(const pg_reads* r, const int64_t* names, const Params& p, int32_t k, int32_t nContigs)
      : R(r), nameId(names), P(p), K(k), strays(names != nullptr) {
    scanStats.bamType = P.bamType;
    cb.assign(nContigs, 0); ce.assign(nContigs, 0); span.assign(nContigs, 1);
    int64_t i = 0;
    for (int32_t c = 0; c < nContigs; c++) {
      while (i < R->n_reads && R->ref_id[i] < c) i++;
      cb[c] = i;
      while (i < R->n_reads && R->ref_id[i] == c) {
        int32_t e = (R->flag[i] & 0x4) ? R->pos[i] : R->aend[i];
        span[c] = std::max(span[c], e - R->pos[i] + 1);
        i++;
      }
      ce[c] = i;
    }
    scan(nContigs);
  }
  void scan(int32_t nContigs) {  // :295-337 (every contig is of interest)
    for (int64_t i = 0; i < R->n_reads; i++) {
      uint16_t fl = R->flag[i];
      if (!validateRead(fl, P) || (fl & 0x4)) continue;
      if (fl & 0x1) {
        if (fl & 0x2) scanStats.addInsert(R->tlen[i], fl & 0x10, false);
        else if (strays && !(fl & 0x8)) {
          bool soi = (R->ref_id[i] >= 0 && R->ref_id[i] < nContigs) ||
                     (R->mate_ref_id[i] >= 0 && R->mate_ref_id[i] < nContigs);
          if (soi) ((fl & 0x40) ? stray1 : stray2)[nameId[i]] = i;
        }
      } else {
        scanStats.addInsert(R->l_seq[i], fl & 0x10, true);
      }
    }
  }
  std::vector<int64_t> readsInRegion(int32_t c, int32_t s, int32_t e) const {  // :339-344
    // queryOverlapping: the alignment [start, end] (end = start when unmapped) meets [s, e]
    const int32_t* pos = R->pos;
    int64_t lo = std::lower_bound(pos + cb[c], pos + ce[c], (int64_t)s - span[c]) - pos;
    int64_t hi = std::upper_bound(pos + cb[c], pos + ce[c], e) - pos;
    std::vector<int64_t> out;
    for (int64_t i = lo; i < hi; i++) {
      int32_t end = (R->flag[i] & 0x4) ? R->pos[i] : R->aend[i];
      if (R->pos[i] <= e && end >= s && validateRead(R->flag[i], P)) out.push_back(i);
    }
    return out;
  }
  // MateMap.findStrays (S/BamFile.scala:244-257) of the MateMap m1 / m2 (name ->
  // read, first-of-pair reads in m1); in HashMap order in the reference, sorted
  // here (the tally and the pairs below do not depend on the order)
  std::vector<int64_t> findStrays(const std::unordered_map<int64_t, int64_t>& m1,
                                  const std::unordered_map<int64_t, int64_t>& m2) const {
    std::vector<int64_t> found;
    for (auto& kv : m1)
      if (!m2.count(kv.first)) { auto it = stray2.find(kv.first); if (it != stray2.end()) found.push_back(it->second); }
    for (auto& kv : m2)
      if (!m1.count(kv.first)) {
        auto& sm = (R->flag[kv.second] & 0x40) ? stray2 : stray1;
        auto it = sm.find(kv.first);
        if (it != sm.end()) found.push_back(it->second);
      }
    std::sort(found.begin(), found.end());
    return found;
  }
  std::vector<int64_t> recruitReads(const BamStats& st, int32_t c, int32_t s, int32_t e) const {
    // GapFiller.recruitReads (S/GapFiller.scala:364-402) for the one BAM
    if (P.bamType == PG_BAM_UNPAIRED && P.longRead) return {};  // recruitUnpaired with --nanopore/--pacbio
    int32_t flank = st.maxInsertSize();
    int32_t fs = std::max(s - flank, 1), fe = e + flank;  // flankRegion (S/BamFile.scala:359-364)
    std::vector<int64_t> reads = readsInRegion(c, fs, fe);
    std::unordered_map<int64_t, int64_t> m1, m2;  // MateMap(reads)
    if (strays || P.bamType == PG_BAM_JUMPS)
      for (int64_t i : reads) ((R->flag[i] & 0x40) ? m1 : m2)[nameId ? nameId[i] : i] = i;
    if (P.bamType == PG_BAM_JUMPS) {  // recruitJumps -> recruitBadMates (S/BamFile.scala:366-403)
      if (strays)
        for (int64_t i : findStrays(m1, m2)) ((R->flag[i] & 0x40) ? m1 : m2)[nameId[i]] = i;  // addStrays
      int32_t midpoint = (s + e) / 2;
      int64_t frPct = st.pctFR();
      std::vector<int64_t> mates;
      for (auto& kv : m1) {  // pairs(): (read1, read2) and (read2, read1) of each name in both maps
        auto it = m2.find(kv.first);
        if (it == m2.end()) continue;
        for (auto [a, b] : {std::pair<int64_t, int64_t>{kv.second, it->second}, {it->second, kv.second}}) {
          uint16_t fl = R->flag[a];
          if ((fl & 0x4) || (fl & 0x2)) continue;
          bool rc = fl & 0x10;
          int32_t st = R->pos[a], en = R->aend[a];
          bool before = st < midpoint, after = en > midpoint;
          bool frO = (before && !rc) || (after && rc);
          bool good = frPct > 100 - 10 ? frO : frPct < 10 ? !frO : true;  // minOrientationPct
          if (good && ((st >= fs && st <= fe) || (en >= fs && en <= fe))) mates.push_back(b);
        }
      }
      std::sort(mates.begin(), mates.end());  // prepended in HashMap order in the reference
      return mates;
    }
    if (strays && P.bamType != PG_BAM_UNPAIRED) {  // recruitFlankReads (S/BamFile.scala:346-357)
      std::vector<int64_t> found = findStrays(m1, m2);
      reads.insert(reads.end(), found.begin(), found.end());
    }
    return reads;
  }
};

void BamStats::addRegion(const GenomeRegion& g) {
  fr.count += g.fr.count; fr.sum += g.fr.sum; fr.sumSq += g.fr.sumSq;
  rf.count += g.rf.count; rf.sum += g.rf.sum; rf.sumSq += g.rf.sumSq;
}

// The K-mer graph walk of one Assembler (S/Assembler.scala:164-284).
struct GraphWalk {
  std::unordered_map<std::string, std::string> kGraph, altGraph;
  int32_t K;
  int32_t loopLength = 0;
  std::string loopSequence;

  // A K-mer path: the reference's List has its newest K-mer at the head; here
  // km is oldest first, with each K-mer's count and latest position.
  struct Path {
    std::vector<std::string> km;
    std::unordered_map<std::string, std::pair<int32_t, int32_t>> at;
    void push(const std::string& k) {
      auto& e = at[k];
      e.first++;
      e.second = (int32_t)km.size();
      km.push_back(k);
    }
    int32_t indexOf(const std::string& k) const {  // List.indexOf from the head
      auto it = at.find(k);
      return it == at.end() ? -1 : (int32_t)km.size() - 1 - it->second.second;
    }
    bool tailContains(const std::string& k) const {  // kmers.tail contains k
      auto it = at.find(k);
      if (it == at.end()) return false;
      return it->second.first - (km.back() == k ? 1 : 0) > 0;
    }
  };

  static std::string pathString(const std::vector<std::string>& km, size_t from) {  // kmerPathString (:164-171)
    std::string s = km[from];
    for (size_t i = from + 1; i < km.size(); i++) s.push_back(km[i].back());
    return s;
  }
  void noteKmerLoop(int32_t loopIndex, const Path& p) {  // :173-181
    int32_t length = loopIndex + 1;
    if (loopLength == 0 || length < loopLength) {
      loopLength = length;
      loopSequence = pathString(p.km, p.km.size() - (size_t)length).substr(0, (size_t)length);
    }
  }
  void pathsForwardFrom(Path p, int32_t branches, std::vector<Path>& out) {  // kmerPathsForward (:183-234)
    while (true) {
      const std::string kmer = p.km.back();
      auto g = kGraph.find(kmer);
      if (g == kGraph.end()) { out.push_back(std::move(p)); return; }
      auto a = altGraph.find(kmer);
      if (a != altGraph.end()) {
        const std::string next1 = g->second, next2 = a->second;
        bool seen1 = p.tailContains(next1), seen2 = p.tailContains(next2);
        if (seen1 || seen2) {
          noteKmerLoop(std::max(p.indexOf(next1), p.indexOf(next2)), p);
          out.push_back(std::move(p));  // trSafe
          return;
        }
        if (branches < 5) {  // maxBranches
          Path p2 = p;
          p.push(next1);
          pathsForwardFrom(std::move(p), branches + 1, out);
          p2.push(next2);
          pathsForwardFrom(std::move(p2), branches + 1, out);
        } else {
          out.push_back(std::move(p));
        }
        return;
      }
      const std::string next = g->second;
      int32_t loop = p.indexOf(next);
      if (loop >= 0) {
        noteKmerLoop(loop, p);
        out.push_back(std::move(p));  // trSafe
        return;
      }
      p.push(next);
    }
  }
  std::vector<std::string> pathsForward(const std::string& start) {  // :236-247
    Path p;
    p.push(start);
    std::vector<Path> kp;
    pathsForwardFrom(std::move(p), 0, kp);
    std::vector<std::string> paths;
    for (auto& q : kp) paths.push_back(pathString(q.km, 0));
    std::stable_sort(paths.begin(), paths.end(), [](const std::string& a, const std::string& b) {
      return a.size() > b.size();
    });
    return paths;
  }
  std::vector<std::string> tryForward(const std::string& anchor) {  // :254-267
    if ((int32_t)anchor.size() < K) return {anchor};
    std::string startingKmer = anchor.substr(0, K);
    std::vector<std::string> paths = pathsForward(startingKmer);
    if (!paths.empty() && paths[0].size() > anchor.size() + 20) return paths;  // minExtend
    std::vector<std::string> out;
    for (auto& p : tryForward(anchor.substr(K))) out.push_back(startingKmer + p);
    return out;
  }
  std::vector<std::string> tryReverse(const std::string& anchor) {  // :269-278
    std::vector<std::string> out;
    for (auto& p : tryForward(revComp(anchor))) out.push_back(revComp(p));
    return out;
  }
};

// properOverlap (S/GapFiller.scala:220-245)
static std::string properOverlap(const std::string& left, const std::string& right, int32_t minOverlap) {
  int32_t ll = (int32_t)left.size(), rl = (int32_t)right.size();
  for (int32_t overlap = minOverlap; overlap <= ll + rl - 2 * minOverlap; overlap++) {
    int32_t lo = std::max(ll - overlap, 0), ro = std::max(overlap - ll, 0);
    int32_t len = std::min(ll - lo, rl - ro);
    bool match = true;
    for (int32_t i = 0; i < len; i++)
      if (left[lo + i] != right[ro + i]) { match = false; break; }
    if (match) return left.substr(0, lo) + right.substr(ro);
  }
  return "";
}

// trimPatch (S/GapFiller.scala:247-262)
static Fix trimPatch(const GenomeRegion& g, int32_t start, std::string patch, int32_t stop) {
  while (start < stop && !patch.empty() && (g.baseAt(start) == patch[0] || g.originalBaseAt(start) == patch[0])) {
    start++;
    patch.erase(0, 1);
  }
  while (start < stop && !patch.empty() &&
         (g.baseAt(stop - 1) == patch.back() || g.originalBaseAt(stop - 1) == patch.back())) {
    stop--;
    patch.pop_back();
  }
  return Fix{start, g.refSubString(start, stop - start), patch, 2};
}

static std::string consensusFromLeft(const std::vector<std::string>& seqs) {  // :102-110
  const std::string& s0 = seqs.front();
  if (seqs.size() == 1) return s0;
  size_t minLength = s0.size();
  for (auto& s : seqs) minLength = std::min(minLength, s.size());
  for (size_t i = 0; i < minLength; i++)
    for (size_t k = 1; k < seqs.size(); k++)
      if (seqs[k][i] != s0[i]) return s0.substr(0, i);
  return s0.substr(0, minLength);
}
static std::string consensusFromRight(const std::vector<std::string>& seqs) {  // :112-123
  const std::string& s0 = seqs.front();
  if (seqs.size() == 1) return s0;
  size_t minLength = s0.size();
  for (auto& s : seqs) minLength = std::min(minLength, s.size());
  for (size_t i = 0; i < minLength; i++)
    for (size_t k = 1; k < seqs.size(); k++) {
      size_t si = seqs[k].size() - 1 - i, s0i = s0.size() - 1 - i;
      if (seqs[k][si] != s0[s0i]) return s0.substr(s0i + 1);
    }
  return s0.substr(s0.size() - minLength);
}

// GapFiller.assembleAcrossBreak (S/GapFiller.scala:49-100) with
// assembleIntoBreak (:125-159) and breakJoins / joinBreak (:161-218).
Fix reassemble(const GenomeRegion& g, const Reassembly& ra, const BamStats& st, int32_t bs, int32_t be, bool isGap,
               int64_t& tiedSets) {
  const Fix noSolution{0, "", "", 2};
  std::vector<int64_t> reads = ra.recruitReads(st, g.contigId, bs, be);
  GraphWalk w;
  w.K = ra.K;
  {
    auto pileups = tallyReads(ra.R, ra.P, reads.data(), (int64_t)reads.size(), ra.K);
    for (auto& kv : pileups) {
      const PileUp& pu = kv.second;
      if (pu.depth() >= 5) {  // Assembler.minDepth
        BaseCall bc = baseCall(pu, ra.P);
        std::string prefix = kv.first.substr(1);
        w.kGraph[kv.first] = prefix + bc.base;
        if (!bc.homo) w.altGraph[kv.first] = prefix + bc.altBase;
      }
    }
  }
  int32_t radius = st.breakRadius(ra.K);
  int32_t start = std::max(bs - radius, g.start);
  int32_t stop = std::min(be + 1 + radius, g.stop);
  std::string left = g.subString(start, bs - start);
  std::string right = g.subString(be + 1, stop - be - 1);
  std::vector<std::string> pathsFromLeft = w.tryForward(left);
  std::vector<std::string> pathsFromRight = w.tryReverse(right);
  const std::string& loop = w.loopSequence;
  // breakJoins: a Set of solutions (insertion order for up to four elements)
  std::vector<Fix> set;
  int32_t k = 2 * ra.K + 1;  // GapFiller.k
  for (auto& f : pathsFromLeft)
    for (auto& r : pathsFromRight) {
      std::string patch = properOverlap(f, r, k);
      if (patch.empty()) continue;
      Fix s = trimPatch(g, start, patch, stop);
      if (std::find(set.begin(), set.end(), s) == set.end()) set.push_back(s);
    }
  std::vector<Fix> solutions = set;
  std::stable_sort(solutions.begin(), solutions.end(), [](const Fix& a, const Fix& b) {
    return a.patch.size() + a.was.size() < b.patch.size() + b.was.size();
  });
  std::vector<int64_t> lengths;
  for (auto& s : set) {
    int64_t d = (int64_t)s.patch.size() - (int64_t)s.was.size();
    if (std::find(lengths.begin(), lengths.end(), d) == lengths.end()) lengths.push_back(d);
  }
  if (lengths.size() == 1) {
    if (set.size() > 4 && solutions.size() > 1 &&
        solutions[1].patch.size() + solutions[1].was.size() == solutions[0].patch.size() + solutions[0].was.size())
      tiedSets++;  // the reference takes the first of a HashSet's order here
    solutions.resize(1);
  }
  Fix solution = solutions.size() == 1 ? solutions[0] : noSolution;
  bool solutionOK = !(solution == noSolution) && loop.empty();
  if (solutionOK && isGap) {
    int64_t closedDiff = std::llabs((int64_t)solution.patch.size() - (int64_t)(be + 1 - bs));
    if (closedDiff > ra.gapMargin) solutionOK = false;  // Pilon.gapMargin
  }
  if (solutionOK) return solution;
  if (!(isGap || (ra.fixBreaks && loop.empty()))) return noSolution;
  std::string fromRight = consensusFromRight(pathsFromRight);
  std::string fromLeft = consensusFromLeft(pathsFromLeft);
  int32_t newStart = start + (int32_t)fromLeft.size();
  int32_t newStop = stop - (int32_t)fromRight.size();
  auto partialMatchesReference = [&]() {  // :264-281
    if (start + (int32_t)fromLeft.size() > g.stop || stop - (int32_t)fromRight.size() < g.start) return false;
    std::string regionLeft = g.subString(start, (int32_t)fromLeft.size());
    std::string regionRight = g.subString(stop - (int32_t)fromRight.size(), (int32_t)fromRight.size());
    return fromLeft == regionLeft && fromRight == regionRight;
  };
  if ((newStart >= bs + 20 || newStop <= be - 20) && !partialMatchesReference()) {  // GapFiller.minExtend
    int32_t newGapLength = isGap ? std::max(ra.minGap, newStop - newStart) : ra.minGap;  // Pilon.minGap
    // (1 to newGapLength) map {_ => "N"}: empty when newGapLength <= 0
    std::string seq = fromLeft + std::string((size_t)std::max(newGapLength, 0), 'N') + fromRight;
    Fix s = trimPatch(g, start, seq, stop);
    return s.patch.empty() ? noSolution : s;
  }
  return noSolution;
}

std::string regionString(const std::string& name, int32_t s, int32_t e) {  // S/Region.scala:45
  int32_t size = e + 1 - s;
  return name + ":" + std::to_string(s) + (size < 2 ? "" : "-" + std::to_string(e));
}

Params toParams(const pg_params* p) {
  Params P;
  P.minMq = p->min_mq; P.minQual = p->min_qual; P.flank = p->flank; P.defaultQual = p->default_qual;
  P.minMinDepth = p->min_min_depth; P.nonPf = p->nonpf; P.duplicates = p->duplicates;
  P.oldIndel = p->old_indel; P.fixAmb = p->fix_amb; P.longRead = p->long_read; P.bamType = p->bam_type;
  P.longReadOnly = p->long_read_only; P.minDepth = p->min_depth;
  return P;
}

void fillOut(GenomeRegion& g, pg_region_out* o, pg_region_stats* st, const Params& P) {
  int32_t n = g.size();
  std::vector<int32_t> insOffsets;
  int64_t charPos = 0;
  int32_t nIns = 0;
  for (int32_t i = 0; i < n; i++) {
    const PileUp& pu = g.pr.pileups[i];
    if (o->count) for (int b = 0; b < 4; b++) o->count[4 * (int64_t)i + b] = (int32_t)pu.baseCount[b];
    if (o->qual_sum) for (int b = 0; b < 4; b++) o->qual_sum[4 * (int64_t)i + b] = pu.qualSum[b];
    if (o->mq_sum) o->mq_sum[i] = pu.mqSum;
    if (o->q_sum) o->q_sum[i] = pu.qSum;
    if (o->phys_cov) o->phys_cov[i] = pu.physCov;
    if (o->insert_size) o->insert_size[i] = pu.insertSize;
    if (o->bad_pair) o->bad_pair[i] = pu.badPair;
    if (o->deletions) o->deletions[i] = pu.deletions;
    if (o->del_qual) o->del_qual[i] = pu.delQual;
    if (o->insertions) o->insertions[i] = pu.insertions;
    if (o->ins_qual) o->ins_qual[i] = pu.insQual;
    if (o->clips) o->clips[i] = pu.clips;
    BaseCall bc = baseCall(pu, P);
    uint32_t f = (uint32_t)bc.baseIdx | ((uint32_t)bc.altIdx << 2);
    if (bc.n > 0) f |= PG_CALL_HAS_BASE;
    if (bc.homo) f |= PG_CALL_HOMO;
    if (bc.isInsertion()) f |= PG_CALL_INS;
    if (bc.isDeletion()) f |= PG_CALL_DEL;
    if (bc.homoIndel) f |= PG_CALL_HOMO_INDEL;
    auto it = g.changeMap.find(i);
    if (it != g.changeMap.end()) f |= ((uint32_t)it->second.first) << 9;
    if (g.confirmed[i]) f |= PG_CALL_CONFIRMED;
    if (g.deleted[i]) f |= PG_CALL_DELETED;
    if (o->call) o->call[i] = f;
    if (o->score) o->score[i] = bc.score;
    int32_t il = bc.isInsertion() ? (int32_t)bc.insertion.size() : bc.isDeletion() ? (int32_t)bc.deletion.size() : 0;
    if (o->indel_len) o->indel_len[i] = il;
    if (o->ins_str) o->ins_str[i] = -1;
    if (bc.isInsertion()) {
      if (o->ins_str) o->ins_str[i] = (int32_t)charPos;
      if (o->ins_chars && charPos + (int64_t)bc.insertion.size() <= o->ins_chars_cap)
        memcpy(o->ins_chars + charPos, bc.insertion.data(), bc.insertion.size());
      charPos += (int64_t)bc.insertion.size();
      nIns++;
    }
  }
  if (st) {
    st->base_count = g.pr.baseCount;
    st->read_count = g.pr.readCount;
    st->phys_cov_start = g.pr.physCovStart;
    st->insert_size_start = g.pr.insertSizeStart;
    st->min_depth = g.minDepth;
    st->n_changes = (int32_t)g.changeMap.size();
    st->fr_count = g.fr.count; st->fr_sum = g.fr.sum; st->fr_sumsq = g.fr.sumSq;
    st->rf_count = g.rf.count; st->rf_sum = g.rf.sum; st->rf_sumsq = g.rf.sumSq;
    st->error = 0;
    st->n_ins_strings = nIns;
  }
}

}  // namespace

extern "C" {

// One region end to end: BamFile.process + postProcess (pass 1 and 2).
// Returns 0, or PG_ERR_INDEX where the reference would throw.
int or_process_region(const pg_reads* R, const pg_params* params, const uint8_t* contig, int64_t contig_len,
                      int32_t contig_id, int32_t start, int32_t stop, int64_t read_begin, int64_t read_end,
                      pg_region_out* out, pg_region_stats* stats) {
  Params P = toParams(params);
  try {
    GenomeRegion g("c", contig_id, contig, contig_len, start, stop, P);
    g.processBam(R, read_begin, read_end);
    g.postProcess();
    fillOut(g, out, stats, P);
  } catch (IndexError&) {
    if (stats) { memset(stats, 0, sizeof *stats); stats->error = PG_ERR_INDEX; }
    return PG_ERR_INDEX;
  }
  return 0;
}

// Contig chunking of GenomeFile.contigRegions (S/GenomeFile.scala:67-74).
// Writes up to cap (start, stop) pairs; returns the number of regions.
int32_t or_contig_regions(int64_t contig_len, int32_t chunk_size, int32_t* starts, int32_t* stops, int32_t cap) {
  int64_t nChunks = (contig_len + chunk_size - 1) / chunk_size;
  int64_t cs = (contig_len + nChunks - 1) / nChunks;
  int32_t n = 0;
  for (int64_t b = 1; b < contig_len + 1; b += cs) {
    if (n < cap) { starts[n] = (int32_t)b; stops[n] = (int32_t)std::min<int64_t>(contig_len, b + cs - 1); }
    n++;
  }
  return n;
}

// Whole-genome polish with --fix snps,indels[,amb] --vcf --changes: the loop of
// GenomeFile.processRegions (S/GenomeFile.scala:84-176) for one BAM, writing the
// FASTA, VCF and changes files the reference writes.  Gap filling and local
// reassembly are not part of this oracle.
static int polishImpl(const pg_reads* R, const pg_params* params, int32_t n_contigs, const char* const* names,
                      const int64_t* lens, const uint8_t* const* bases, int32_t chunk_size, int32_t fix_snps,
                      int32_t fix_indels, int32_t iupac, int32_t diploid, int32_t vcf_qe, const char* fasta_path,
                      const char* vcf_path, const char* changes_path, const char* vcf_date, const char* vcf_source,
                      const char* vcf_args, const char* vcf_ref, int32_t fix_gaps, int32_t fix_local, int32_t K,
                      const int64_t* name_id, int64_t* tied_sets, int32_t fix_breaks, int32_t gap_margin,
                      int32_t min_gap) {
  Params P = toParams(params);
  // a BAM of type "bam" is typed by autoBam during the scan, which this oracle does not restate
  if ((fix_gaps || fix_local) && P.bamType == PG_BAM_BAM) return PG_ERR_ARG;
  try {
    // BamFile.scan runs first when strays are tracked (S/GenomeFile.scala:89-92)
    std::unique_ptr<Reassembly> ra;
    if (fix_gaps || fix_local) {
      ra.reset(new Reassembly(R, name_id, P, K, n_contigs));
      ra->fixBreaks = fix_breaks != 0;
      ra->gapMargin = gap_margin;
      ra->minGap = min_gap;
    }
    // region read ranges: reads are sorted by (ref_id, pos); take each contig's span
    std::vector<int64_t> cb(n_contigs, 0), ce(n_contigs, 0);
    {
      int64_t i = 0;
      for (int32_t c = 0; c < n_contigs; c++) {
        while (i < R->n_reads && R->ref_id[i] < c) i++;
        cb[c] = i;
        while (i < R->n_reads && R->ref_id[i] == c) i++;
        ce[c] = i;
      }
    }
    std::vector<std::vector<GenomeRegion*>> regs(n_contigs);
    for (int32_t c = 0; c < n_contigs; c++) {
      int64_t nChunks = (lens[c] + chunk_size - 1) / chunk_size;
      int64_t cs = (lens[c] + nChunks - 1) / nChunks;
      for (int64_t b = 1; b < lens[c] + 1; b += cs)
        regs[c].push_back(new GenomeRegion(names[c], c, bases[c], lens[c], (int32_t)b,
                                           (int32_t)std::min<int64_t>(lens[c], b + cs - 1), P));
    }
    // GenomeFile.processRegions takes the regions one after another; a region's
    // pileups do not depend on the others, and its reassembly reads the
    // insert statistics of the scan and of the regions up to it, so the
    // regions run on all host threads with those statistics taken in order.
    std::vector<GenomeRegion*> flat;
    for (auto& v : regs) flat.insert(flat.end(), v.begin(), v.end());
    auto parallel = [&](auto&& body) {
      std::atomic<size_t> next{0};
      std::atomic<bool> failed{false};
      auto work = [&]() {
        for (size_t k; (k = next.fetch_add(1)) < flat.size();) {
          try {
            body(k);
          } catch (IndexError&) {
            failed = true;
          }
        }
      };
      unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)flat.size()));
      std::vector<std::thread> th;
      for (unsigned t = 1; t < nt; t++) th.emplace_back(work);
      work();
      for (auto& t : th) t.join();
      if (failed) throw IndexError();
    };
    parallel([&](size_t k) {
      GenomeRegion* g = flat[k];
      g->processBam(R, cb[g->contigId], ce[g->contigId]);
      g->postProcess();
    });
    std::vector<BamStats> seen(flat.size());
    if (ra) {
      BamStats acc = ra->scanStats;
      for (size_t k = 0; k < flat.size(); k++) {
        acc.addRegion(*flat[k]);
        seen[k] = acc;
      }
    }
    parallel([&](size_t k) {
      flat[k]->identifyAndFixIssues(fix_snps, fix_indels, iupac, P.longRead != 0, ra.get(), &seen[k], fix_gaps,
                                    fix_local);
    });
    if (tied_sets) {
      *tied_sets = 0;
      for (auto* g : flat) *tied_sets += g->tiedSets;
    }
    FILE* fc = changes_path ? fopen(changes_path, "w") : nullptr;
    FILE* ff = fasta_path ? fopen(fasta_path, "w") : nullptr;
    FILE* fv = vcf_path ? fopen(vcf_path, "w") : nullptr;
    VcfWriter vw{fv, (bool)diploid, (bool)vcf_qe, P};
    if (fv) {
      std::vector<std::pair<std::string, int64_t>> cs;
      for (int32_t c = 0; c < n_contigs; c++) {
        int64_t s = 0;
        for (auto* g : regs[c]) s += g->size();
        cs.push_back({names[c], s});
      }
      vw.header(cs, vcf_date, vcf_source, vcf_args, vcf_ref);
    }
    for (int32_t c = 0; c < n_contigs; c++) {
      std::string name = names[c];
      std::string sep = name.find('|') == std::string::npos ? "_" : (name.back() == '|' ? "" : "|");
      std::string newName = name + sep + "pilon";
      int32_t offset = 0;
      for (auto* g : regs[c]) {
        if (fv) vw.writeRegion(*g);
        if (fc) {  // writeChanges (S/GenomeRegion.scala:645-657)
          int32_t delta = 0;
          for (auto& fx : g->allFixes()) {
            int32_t newLoc = fx.locus + delta;
            std::string o = regionString(g->name, fx.locus, fx.locus + (int32_t)fx.was.size() - 1);
            std::string nw = regionString(newName, newLoc + offset, newLoc + offset + (int32_t)fx.patch.size() - 1);
            fprintf(fc, "%s %s %s %s\n", o.c_str(), nw.c_str(), fx.was.empty() ? "." : fx.was.c_str(),
                    fx.patch.empty() ? "." : fx.patch.c_str());
            delta += (int32_t)fx.patch.size() - (int32_t)fx.was.size();
          }
          offset += (int32_t)g->bases.size() - g->size();
        }
      }
      if (ff) {  // writeFastaElement (S/GenomeFile.scala:79-82)
        std::string seq;
        for (auto* g : regs[c]) seq.append(g->bases.begin(), g->bases.end());
        fprintf(ff, ">%s\n", newName.c_str());
        for (size_t k = 0; k < seq.size(); k += 80) {
          fwrite(seq.data() + k, 1, std::min<size_t>(80, seq.size() - k), ff);
          fputc('\n', ff);
        }
      }
    }
    if (fc) fclose(fc);
    if (ff) fclose(ff);
    if (fv) fclose(fv);
    for (auto& v : regs) for (auto* g : v) delete g;
  } catch (IndexError&) {
    return PG_ERR_INDEX;
  }
  return 0;
}

}  // extern "C"

extern "C" {

// Whole-genome polish (GenomeFile.processRegions, S/GenomeFile.scala:84-176)
// with --fix snps,indels[,amb] --vcf --changes.
int or_polish(const pg_reads* R, const pg_params* params, int32_t n_contigs, const char* const* names,
              const int64_t* lens, const uint8_t* const* bases, int32_t chunk_size, int32_t fix_snps,
              int32_t fix_indels, int32_t iupac, int32_t diploid, int32_t vcf_qe, const char* fasta_path,
              const char* vcf_path, const char* changes_path, const char* vcf_date, const char* vcf_source,
              const char* vcf_args, const char* vcf_ref) {
  return polishImpl(R, params, n_contigs, names, lens, bases, chunk_size, fix_snps, fix_indels, iupac, diploid,
                    vcf_qe, fasta_path, vcf_path, changes_path, vcf_date, vcf_source, vcf_args, vcf_ref, 0, 0, 31,
                    nullptr, nullptr, 0, 100000, 10);
}

// The same with the fix types gaps and local as well (GapFiller fillGap /
// fixBreak, S/GenomeRegion.scala:382-410): K is Assembler.K (--K), name_id the
// read name of each read as an id (mates share one; NULL: no stray mates, as
// --nostrays), fix_breaks the experimental "breaks" fix (--variant),
// gap_margin and min_gap Pilon's --gapmargin and --mingap.
// *tied_sets receives the count of solution sets of more than four elements
// whose first element had to be taken in an order the reference gets from its
// HashSet (see reassemble).
int or_polish_fix(const pg_reads* R, const pg_params* params, int32_t n_contigs, const char* const* names,
                  const int64_t* lens, const uint8_t* const* bases, int32_t chunk_size, int32_t fix_snps,
                  int32_t fix_indels, int32_t iupac, int32_t diploid, int32_t vcf_qe, const char* fasta_path,
                  const char* vcf_path, const char* changes_path, const char* vcf_date, const char* vcf_source,
                  const char* vcf_args, const char* vcf_ref, int32_t fix_gaps, int32_t fix_local, int32_t K,
                  const int64_t* name_id, int64_t* tied_sets, int32_t fix_breaks, int32_t gap_margin,
                  int32_t min_gap) {
  return polishImpl(R, params, n_contigs, names, lens, bases, chunk_size, fix_snps, fix_indels, iupac, diploid,
                    vcf_qe, fasta_path, vcf_path, changes_path, vcf_date, vcf_source, vcf_args, vcf_ref, fix_gaps,
                    fix_local, K, name_id, tied_sets, fix_breaks, gap_margin, min_gap);
}

// One --targets region end to end (S/GenomeFile.scala:215-250): processBam,
// postProcess, identifyAndFixIssues; writes the fixed bases (no header, no line
// breaks), the region's changes lines (the target is its own output entry, so
// the offset is 0) and the region's VCF records (GenomeRegion.writeVcf, no
// header).  Returns 0, or PG_ERR_INDEX where the reference would throw.
int or_target(const pg_reads* R, const pg_params* params, const char* name, const uint8_t* contig, int64_t contig_len,
              int32_t contig_id, int32_t start, int32_t stop, int64_t rb, int64_t re, int32_t fix_snps,
              int32_t fix_indels, int32_t iupac, int32_t diploid, int32_t vcf_qe, const char* bases_path,
              const char* changes_path, const char* vcf_path) {
  Params P = toParams(params);
  try {
    GenomeRegion g(name, contig_id, contig, contig_len, start, stop, P);
    g.processBam(R, rb, re);
    g.postProcess();
    g.identifyAndFixIssues(fix_snps, fix_indels, iupac, P.longRead != 0);
    std::string nm = name;
    std::string sep = nm.find('|') == std::string::npos ? "_" : (nm.back() == '|' ? "" : "|");
    std::string newName = nm + sep + "pilon";
    if (FILE* fb = bases_path ? fopen(bases_path, "wb") : nullptr) {
      fwrite(g.bases.data(), 1, g.bases.size(), fb);
      fclose(fb);
    }
    if (FILE* fc = changes_path ? fopen(changes_path, "w") : nullptr) {
      int32_t delta = 0;
      for (auto& fx : g.allFixes()) {
        int32_t newLoc = fx.locus + delta;
        std::string o = regionString(g.name, fx.locus, fx.locus + (int32_t)fx.was.size() - 1);
        std::string nw = regionString(newName, newLoc, newLoc + (int32_t)fx.patch.size() - 1);
        fprintf(fc, "%s %s %s %s\n", o.c_str(), nw.c_str(), fx.was.empty() ? "." : fx.was.c_str(),
                fx.patch.empty() ? "." : fx.patch.c_str());
        delta += (int32_t)fx.patch.size() - (int32_t)fx.was.size();
      }
      fclose(fc);
    }
    if (FILE* fv = vcf_path ? fopen(vcf_path, "w") : nullptr) {
      VcfWriter vw{fv, (bool)diploid, (bool)vcf_qe, P};
      vw.writeRegion(g);
      fclose(fv);
    }
  } catch (IndexError&) {
    return PG_ERR_INDEX;
  }
  return 0;
}

// Break candidates of one region (possibleBreaks, S/GenomeRegion.scala:719-720),
// after process + postProcess.  Writes (start, stop) loci; returns the count.
int32_t or_region_breaks(const pg_reads* R, const pg_params* params, const uint8_t* contig, int64_t contig_len,
                         int32_t contig_id, int32_t start, int32_t stop, int64_t rb, int64_t re, int32_t* out,
                         int32_t cap) {
  Params P = toParams(params);
  try {
    GenomeRegion g("c", contig_id, contig, contig_len, start, stop, P);
    g.processBam(R, rb, re);
    g.postProcess();
    auto br = g.possibleBreaks();
    for (size_t k = 0; k < br.size() && (int32_t)k < cap; k++) { out[2 * k] = br[k].first; out[2 * k + 1] = br[k].second; }
    return (int32_t)br.size();
  } catch (IndexError&) {
    return -PG_ERR_INDEX;
  }
}

}  // extern "C"

// Assembler.addReads + buildGraph (S/Assembler.scala:46-87, 132-162) for each
// window; emit(window, K-mer string, its pileup, its call) for every K-mer of
// depth >= min_depth, in (window, K-mer string) order.
template <class Emit>
static void tally_windows(const pg_reads* R, const Params& P, const pg_window* wins, int32_t n_wins, int32_t K,
                          int32_t min_depth, Emit emit) {
  for (int32_t w = 0; w < n_wins; w++) {
    std::unordered_map<std::string, PileUp> pileups;
    int64_t nReads = 0;
    auto addToPileups = [&](const std::string& b, const std::vector<int32_t>& q, int32_t mq) {
      int32_t length = (int32_t)b.size();
      for (int32_t off = 0; off <= length - K - 1; off++) {
        PileUp& pu = pileups[b.substr(off, K)];
        pu.add(b[off + K], q[off + K], mq, P);
      }
    };
    for (int64_t i = wins[w].read_begin; i < wins[w].read_end; i++) {
      ReadView rv{R, i};
      std::string b = rv.length() > 0 ? rv.bases() : std::string("*");
      int32_t length = (int32_t)b.size();
      if (length > K) {
        std::vector<int32_t> q(length);
        for (int32_t k = 0; k < length; k++) q[k] = rv.qual(k, P);
        int32_t mq = rv.mq();
        addToPileups(b, q, mq);
        std::string rc(b.rbegin(), b.rend());
        for (auto& c : rc) c = c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : c == 'T' ? 'A' : c;
        std::vector<int32_t> rq(q.rbegin(), q.rend());
        addToPileups(rc, rq, mq);
        nReads++;
        if (nReads % 100000 == 0) {  // prunePileups(2)
          for (auto it = pileups.begin(); it != pileups.end();)
            if (it->second.count() < 2) it = pileups.erase(it); else ++it;
        }
      }
    }
    std::vector<std::string> ks;
    for (auto& kv : pileups)
      if (kv.second.depth() >= min_depth) ks.push_back(kv.first);
    std::sort(ks.begin(), ks.end());
    for (auto& k : ks) {
      const PileUp& pu = pileups[k];
      emit(w, k, pu, baseCall(pu, P));
    }
  }
}

static uint64_t nib_of(char c) { return (uint64_t)(strchr(kNib, c) - kNib); }

extern "C" {

// The tally of tally_windows for K <= 32: K-mers as 4-bit BAM codes, base j at
// nibble (15 - j%16) of word j/16.
int64_t or_kmer_tally(const pg_reads* R, const pg_params* params, const pg_window* wins, int32_t n_wins, int32_t K,
                      int32_t min_depth, pg_kmer_edge* edges, int64_t cap) {
  Params P = toParams(params);
  int64_t ne = 0;
  tally_windows(R, P, wins, n_wins, K, min_depth, [&](int32_t w, const std::string& k, const PileUp& pu,
                                                      const BaseCall& bc) {
    if (ne < cap) {
      uint64_t hi = 0, lo = 0;
      for (int32_t j = 0; j < K; j++) {
        if (j < 16) hi |= nib_of(k[j]) << (60 - 4 * j); else lo |= nib_of(k[j]) << (60 - 4 * (j - 16));
      }
      pg_kmer_edge& e = edges[ne];
      e.key_hi = hi;
      e.key_lo = lo;
      e.window = w;
      e.next = (int8_t)bc.baseIdx;
      e.alt = bc.homo ? (int8_t)-1 : (int8_t)bc.altIdx;
      e.pad_ = 0;
      e.depth = (int32_t)pu.depth();
      e.weight = (int32_t)pu.baseCount[bc.baseIdx];
    }
    ne++;
  });
  return ne;
}

// The same tally for any K <= 64 (the reference's K is unbounded; its default
// is 47, S/Assembler.scala:25): base j at bits 60 - 4 (j % 16) of key[j / 16].
int64_t or_kmer_tally_wide(const pg_reads* R, const pg_params* params, const pg_window* wins, int32_t n_wins,
                           int32_t K, int32_t min_depth, pg_kmer_edge_wide* edges, int64_t cap) {
  Params P = toParams(params);
  int64_t ne = 0;
  tally_windows(R, P, wins, n_wins, K, min_depth, [&](int32_t w, const std::string& k, const PileUp& pu,
                                                      const BaseCall& bc) {
    if (ne < cap) {
      pg_kmer_edge_wide& e = edges[ne];
      memset(&e, 0, sizeof e);
      for (int32_t j = 0; j < K && j < 64; j++) e.key[j / 16] |= nib_of(k[j]) << (60 - 4 * (j % 16));
      e.window = w;
      e.next = (int8_t)bc.baseIdx;
      e.alt = bc.homo ? (int8_t)-1 : (int8_t)bc.altIdx;
      e.depth = (int32_t)pu.depth();
      e.weight = (int32_t)pu.baseCount[bc.baseIdx];
    }
    ne++;
  });
  return ne;
}

// Java "%.2f" of a double (exposed for the known-answer tests).
int or_java_format2(double x, char* buf, int cap) {
  std::string s = javaFormat2(x);
  if ((int)s.size() + 1 > cap) return -1;
  memcpy(buf, s.c_str(), s.size() + 1);
  return (int)s.size();
}

}  // extern "C"
