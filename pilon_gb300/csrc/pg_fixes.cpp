// pg_fixes.cpp — the host side of a region's fixes: the fix lists Pilon's
// GenomeRegion.identifyAndFixIssues builds from the pass-1 changes
// (S/GenomeRegion.scala:307-380), fixFixList and fixIssues
// (S/GenomeRegion.scala:557-621), and the changes file's lines
// (S/GenomeRegion.scala:645-657, S/GenomeFile.scala:150-161).
//
// The device compacts the changes (pg_fetch_changes); what is left per change
// is a few string operations, which a polishing run does once per change
// (1.3 million on a 133 Mb draft at 1% variants).  Done here in C++ they no
// longer dominate the run's wall clock.  No context and no device are used.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pilon_gb300.h"
#include "pg_host_guard.h"

namespace {

struct Fix {
  int32_t locus;
  int32_t list;
  std::string was, patch;
};

const char kACGT[] = "ACGT";

// Bases.toIUPAC (S/Bases.scala:85-88): the code of the set of two bases, by bit mask A=1 C=2 G=4 T=8.
char iupac(int mask) {
  static const char code[16] = {'?', 'A', 'C', 'M', 'G', 'R', 'S', 'V', 'T', 'W', 'Y', 'H', 'K', 'D', 'B', 'N'};
  return code[mask & 15];
}

char upper(uint8_t b) { return (b >= 'a' && b <= 'z') ? (char)(b - 32) : (char)b; }

// GenomeRegion.fixFixList (S/GenomeRegion.scala:557-593): stable sort by locus, then of two
// overlapping neighbours keep the one with more bases (the first on a tie).
std::vector<const Fix*> fixFixList(const std::vector<const Fix*>& in) {
  std::vector<const Fix*> fx(in);
  std::stable_sort(fx.begin(), fx.end(), [](const Fix* a, const Fix* b) { return a->locus < b->locus; });
  std::vector<const Fix*> out;
  out.reserve(fx.size());
  size_t k = 0;
  while (k < fx.size()) {
    if (k + 1 < fx.size()) {
      const Fix* f1 = fx[k];
      const Fix* f2 = fx[k + 1];
      const int64_t e1 = (int64_t)f1->locus + std::max<int64_t>((int64_t)f1->was.size() - 1, 0);
      const int64_t e2 = (int64_t)f2->locus + std::max<int64_t>((int64_t)f2->was.size() - 1, 0);
      if (f2->locus <= e1 && e2 >= f1->locus) {
        if (f1->was.size() + f1->patch.size() >= f2->was.size() + f2->patch.size()) fx[k + 1] = f1;
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

// GenomeRegion.fixIssues (S/GenomeRegion.scala:595-621): the fixes applied from the last locus
// to the first, each on the original coordinates of `bases` (region loci start..).
std::string fixIssues(const std::string& bases, int32_t start, const std::vector<const Fix*>& fixes) {
  const std::vector<const Fix*> fx = fixFixList(fixes);
  bool ordered = true;  // fixFixList leaves ranges that follow one another: one pass joins them
  int64_t at = 0;
  for (const Fix* f : fx) {
    const int64_t s = (int64_t)f->locus - start;
    if (s < at || s > (int64_t)bases.size()) {
      ordered = false;
      break;
    }
    at = s + (int64_t)f->was.size();
  }
  if (ordered) {
    std::string out;
    out.reserve(bases.size() + 64);
    at = 0;
    for (const Fix* f : fx) {
      const int64_t s = (int64_t)f->locus - start;
      out.append(bases, (size_t)at, (size_t)(s - at));
      out += f->patch;
      at = std::min<int64_t>(s + (int64_t)f->was.size(), (int64_t)bases.size());
    }
    out.append(bases, (size_t)at, std::string::npos);
    return out;
  }
  // otherwise one at a time from the last, with slice bounds clamped as a slice of the region's
  // bases is (a fix before the region's start is refused by the caller)
  std::string nb = bases;
  for (auto it = fx.rbegin(); it != fx.rend(); ++it) {
    const Fix* f = *it;
    const int64_t n = (int64_t)nb.size();
    const int64_t s = std::min<int64_t>((int64_t)f->locus - start, n);
    const int64_t e = std::min<int64_t>(s + (int64_t)f->was.size(), n);
    if (f->was.size() == f->patch.size()) {
      nb.replace((size_t)s, (size_t)std::min<int64_t>((int64_t)f->patch.size(), n - s), f->patch);
    } else {
      nb = nb.substr(0, (size_t)s) + f->patch + nb.substr((size_t)e);
    }
  }
  return nb;
}

void regionString(std::string& out, const char* name, int64_t s, int64_t e) {  // Region.regionString (S/Region.scala:45)
  char buf[48];
  out += name;
  int n = e + 1 - s < 2 ? std::snprintf(buf, sizeof buf, ":%lld", (long long)s)
                        : std::snprintf(buf, sizeof buf, ":%lld-%lld", (long long)s, (long long)e);
  out.append(buf, (size_t)n);
}

}  // namespace

extern "C" {

pg_status pg_region_fixes(const pg_change* changes, int64_t n_changes, const char* ins_chars, int64_t n_ins_chars,
                          const uint8_t* contig, int64_t contig_len, int32_t start, int32_t stop,
                          const pg_fix_options* opts, const uint8_t* excluded, pg_fix* fixes, int64_t fix_cap,
                          int64_t* n_fixes, char* text, int64_t text_cap, int64_t* text_len, uint8_t* bases_snp,
                          uint8_t* bases, int64_t bases_cap, int64_t* bases_len) try {
  if (n_changes < 0 || (n_changes > 0 && !changes) || n_ins_chars < 0 || (n_ins_chars > 0 && !ins_chars) ||
      !contig || start < 1 || stop < start || stop > contig_len || !opts || !n_fixes || !text_len || !bases_len ||
      fix_cap < 0 || (fix_cap > 0 && !fixes) || text_cap < 0 || (text_cap > 0 && !text) || !bases_snp ||
      bases_cap < 0 || (bases_cap > 0 && !bases))
    return PG_ERR_ARG;
  const int64_t size = (int64_t)stop - start + 1;
  std::vector<Fix> all;
  all.reserve((size_t)n_changes);
  const bool amb = opts->fix_snps && !opts->long_read;
  for (int64_t i = 0; i < n_changes; i++) {
    const pg_change& c = changes[i];
    const int64_t loc = c.locus;
    if (loc < start || loc > stop) return PG_ERR_ARG;
    if (excluded && excluded[loc - start]) continue;
    const uint32_t f = c.call;
    const int32_t k = (int32_t)((f >> 9) & 7);
    const char cb = (f & PG_CALL_HAS_BASE) ? kACGT[f & 3] : 'N';
    const std::string rb(1, upper(contig[loc - 1]));
    if (k == PG_CHANGE_SNP) {
      if (opts->fix_snps) all.push_back({(int32_t)loc, 0, rb, std::string(1, cb)});
    } else if (k == PG_CHANGE_AMB) {
      if (amb) {
        if (opts->iupac) {
          if (cb == 'N') return PG_ERR_ARG;  // an ambiguous change always has a called base
          const int mask = (1 << (f & 3)) | (1 << ((f >> 2) & 3));
          all.push_back({(int32_t)loc, 1, rb, std::string(1, iupac(mask))});
        } else {
          all.push_back({(int32_t)loc, 0, rb, std::string(1, cb)});
        }
      }
    } else if (k == PG_CHANGE_INS) {
      if (opts->fix_indels) {
        if (c.ins_str < 0 || c.indel_len < 0 || (int64_t)c.ins_str + c.indel_len > n_ins_chars) return PG_ERR_ARG;
        all.push_back({(int32_t)loc, 1, std::string(), std::string(ins_chars + c.ins_str, (size_t)c.indel_len)});
      }
    } else if (k == PG_CHANGE_DEL) {
      if (opts->fix_indels) {
        if (c.indel_len < 0) return PG_ERR_ARG;
        const int64_t e = std::min<int64_t>(loc - 1 + c.indel_len, contig_len);  // a slice of the contig
        all.push_back({(int32_t)loc, 1, std::string((const char*)contig + loc - 1, (size_t)(e - (loc - 1))),
                       std::string()});
      }
    }
  }
  // each list as the reference holds it: prepended, so the last change first
  std::vector<const Fix*> snp, small;
  for (auto it = all.rbegin(); it != all.rend(); ++it) (it->list == 0 ? snp : small).push_back(&*it);
  const std::string orig((const char*)contig + start - 1, (size_t)size);
  const std::string after_snp = fixIssues(orig, start, snp);
  const std::string after_small = fixIssues(after_snp, start, small);
  std::memcpy(bases_snp, after_snp.data(), (size_t)size);  // SNP fixes keep the length
  *bases_len = (int64_t)after_small.size();
  *n_fixes = (int64_t)(snp.size() + small.size());
  int64_t tl = 0;
  for (const Fix* f : snp) tl += (int64_t)(f->was.size() + f->patch.size());
  for (const Fix* f : small) tl += (int64_t)(f->was.size() + f->patch.size());
  *text_len = tl;
  if (*n_fixes > fix_cap || tl > text_cap || *bases_len > bases_cap) return PG_ERR_LIMIT;
  std::memcpy(bases, after_small.data(), after_small.size());
  int64_t k = 0, off = 0;
  for (const std::vector<const Fix*>* list : {&snp, &small}) {
    for (const Fix* f : *list) {
      pg_fix& o = fixes[k++];
      o.locus = f->locus;
      o.list = f->list;
      o.was_off = off;
      o.was_len = (int64_t)f->was.size();
      std::memcpy(text + off, f->was.data(), f->was.size());
      off += o.was_len;
      o.patch_off = off;
      o.patch_len = (int64_t)f->patch.size();
      std::memcpy(text + off, f->patch.data(), f->patch.size());
      off += o.patch_len;
    }
  }
  return PG_OK;
} PG_HOST_CATCH(nullptr)

pg_status pg_changes_lines(const pg_fix* fixes, int64_t n_fixes, const char* text, int64_t text_len,
                           const char* name, const char* new_name, int64_t offset, char* out, int64_t cap,
                           int64_t* out_len) try {
  if (n_fixes < 0 || (n_fixes > 0 && (!fixes || !text)) || text_len < 0 || !name || !new_name || cap < 0 ||
      (cap > 0 && !out) || !out_len)
    return PG_ERR_ARG;
  std::vector<Fix> all((size_t)n_fixes);
  std::vector<const Fix*> ptr((size_t)n_fixes);
  for (int64_t i = 0; i < n_fixes; i++) {
    const pg_fix& f = fixes[i];
    if (f.was_off < 0 || f.was_len < 0 || f.was_off + f.was_len > text_len || f.patch_off < 0 || f.patch_len < 0 ||
        f.patch_off + f.patch_len > text_len)
      return PG_ERR_ARG;
    all[i] = {f.locus, f.list, std::string(text + f.was_off, (size_t)f.was_len),
              std::string(text + f.patch_off, (size_t)f.patch_len)};
    ptr[i] = &all[i];
  }
  std::string lines;
  lines.reserve((size_t)n_fixes * 48);
  int64_t delta = 0;
  for (const Fix* f : fixFixList(ptr)) {
    const int64_t lw = (int64_t)f->was.size(), lp = (int64_t)f->patch.size();
    const int64_t nl = f->locus + delta + offset;
    regionString(lines, name, f->locus, f->locus + lw - 1);
    lines += ' ';
    regionString(lines, new_name, nl, nl + lp - 1);
    lines += ' ';
    lines += lw ? f->was : std::string(".");
    lines += ' ';
    lines += lp ? f->patch : std::string(".");
    lines += '\n';
    delta += lp - lw;
  }
  *out_len = (int64_t)lines.size();
  if (*out_len > cap) return PG_ERR_LIMIT;
  std::memcpy(out, lines.data(), lines.size());
  return PG_OK;
} PG_HOST_CATCH(nullptr)

}  // extern "C"
