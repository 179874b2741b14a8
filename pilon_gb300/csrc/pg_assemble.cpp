// pg_assemble.cpp — local reassembly on the host over the K-mer graphs the
// device tally builds (pg_kmer_tally_reads): the graph walk of Pilon's
// Assembler (S/Assembler.scala:164-284) and the GapFiller that turns the walks
// from both sides of a gap or break into one fix (S/GapFiller.scala:49-262).
//
// The walk is sequential per window, branchy and small, so it stays on the
// CPU; windows run in parallel on host threads.  A window's graph is an
// open-addressing table keyed by the K-mer's 4-bit codes (four 64-bit words,
// K <= 63, as in pg_kmer_edge_wide) holding the called next base and the alt
// base.  A path keeps its K-mers in order with, per K-mer, how often it occurs
// and where it last occurred, so the List.contains / List.indexOf tests of the
// reference walk take constant time.  Pilon.trSafe is always true there, so a
// walk that meets a K-mer it has seen stops; multiClosure and fixNovel are off
// (their defaults); fixBreaks is a field of each job.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "pilon_gb300.h"
#include "pg_host_guard.h"

namespace {

const char kNib[] = "=ACMGRSVTWYHKDBN";
const char kBase[] = "ACGT";

struct Key {
  uint64_t w[4];
  bool operator==(const Key& o) const { return w[0] == o.w[0] && w[1] == o.w[1] && w[2] == o.w[2] && w[3] == o.w[3]; }
};

inline uint64_t mix(uint64_t x) {
  x ^= x >> 31; x *= 0x7fb5d329728ea185ull; x ^= x >> 27; x *= 0x81dadef4bc2dd44dull; x ^= x >> 33;
  return x;
}
inline uint64_t hashKey(const Key& k) { return mix(k.w[0] ^ mix(k.w[1] ^ mix(k.w[2] ^ mix(k.w[3])))); }

int nibOf(char c) {
  const char* p = c ? strchr(kNib, c) : nullptr;
  return p ? (int)(p - kNib) : -1;
}

// The K-mer after `k`: drop its first base, append code `nib` at position K-1.
inline Key advance(const Key& k, int K, int nib) {
  Key n;
  for (int q = 0; q < 3; q++) n.w[q] = (k.w[q] << 4) | (k.w[q + 1] >> 60);
  n.w[3] = k.w[3] << 4;
  const int j = K - 1;
  n.w[j >> 4] |= (uint64_t)nib << (60 - 4 * (j & 15));
  return n;
}

// Open-addressing map Key -> V (no removal).
template <class V>
struct KeyMap {
  std::vector<Key> keys;
  std::vector<V> vals;
  std::vector<uint8_t> used;
  size_t n = 0, mask = 0;
  explicit KeyMap(size_t expect = 16) { rehash(std::max<size_t>(16, expect * 2)); }
  void rehash(size_t cap) {
    size_t c = 16;
    while (c < cap) c <<= 1;
    std::vector<Key> ok;
    std::vector<V> ov;
    std::vector<uint8_t> ou;
    ok.swap(keys); ov.swap(vals); ou.swap(used);
    keys.assign(c, Key{{0, 0, 0, 0}}); vals.assign(c, V()); used.assign(c, 0);
    mask = c - 1;
    n = 0;
    for (size_t i = 0; i < ou.size(); i++)
      if (ou[i]) *insert(ok[i]) = ov[i];
  }
  V* find(const Key& k) {
    for (size_t h = hashKey(k) & mask;; h = (h + 1) & mask) {
      if (!used[h]) return nullptr;
      if (keys[h] == k) return &vals[h];
    }
  }
  const V* find(const Key& k) const { return const_cast<KeyMap*>(this)->find(k); }
  V* insert(const Key& k) {  // the slot of k, added with V() when absent
    if (2 * (n + 1) > keys.size()) rehash(2 * keys.size());
    for (size_t h = hashKey(k) & mask;; h = (h + 1) & mask) {
      if (!used[h]) {
        used[h] = 1; keys[h] = k; n++;
        return &vals[h];
      }
      if (keys[h] == k) return &vals[h];
    }
  }
};

// One window's graph: kGraph (next) and altGraph (alt) of Assembler.buildGraph.
struct Edge {
  int8_t next = -1, alt = -1;
};

struct Graph {
  KeyMap<Edge> g;
  int K;
  explicit Graph(int k, size_t n) : g(n), K(k) {}
};

// A K-mer path in walk order: the K-mers, and per K-mer its count and latest position.
struct Path {
  std::vector<Key> km;
  std::string str;  // kmerPathString: the first K-mer, then each later K-mer's last base
  KeyMap<std::pair<int32_t, int32_t>> at;
  Path() : at(64) {}
  void push(const Key& k, char last) {
    auto* e = at.insert(k);
    e->first++;
    e->second = (int32_t)km.size();
    km.push_back(k);
    str.push_back(last);
  }
  int32_t indexOf(const Key& k) const {  // List.indexOf, counted from the newest K-mer
    const auto* e = at.find(k);
    return e ? (int32_t)km.size() - 1 - e->second : -1;
  }
  bool tailContains(const Key& k) const {  // the List's tail: every K-mer but the newest
    const auto* e = at.find(k);
    return e && e->first - (km.back() == k ? 1 : 0) > 0;
  }
};

struct Walker {
  const Graph& G;
  int K;
  int32_t loopLength = 0;  // Assembler.loopLength: the shortest loop noted so far

  void noteLoop(int32_t loopIndex) {  // Assembler.noteKmerLoop (S/Assembler.scala:173-181)
    const int32_t length = loopIndex + 1;
    if (loopLength == 0 || length < loopLength) loopLength = length;
  }

  // Assembler.kmerPathsForward (S/Assembler.scala:183-234)
  void forward(Path p, int branches, std::vector<std::string>& out) {
    while (true) {
      const Key kmer = p.km.back();
      const Edge* e = G.g.find(kmer);
      if (!e || e->next < 0) { out.push_back(std::move(p.str)); return; }  // end of the line
      const Key n1 = advance(kmer, K, 1 << e->next);
      if (e->alt >= 0) {  // two choices forward
        const Key n2 = advance(kmer, K, 1 << e->alt);
        const bool seen1 = p.tailContains(n1), seen2 = p.tailContains(n2);
        if (seen1 || seen2) {  // a loop: the walk stops there (trSafe)
          noteLoop(std::max(p.indexOf(n1), p.indexOf(n2)));
          out.push_back(std::move(p.str));
          return;
        }
        if (branches < 5) {  // Assembler.maxBranches
          Path q = p;
          p.push(n1, kBase[e->next]);
          forward(std::move(p), branches + 1, out);
          q.push(n2, kBase[e->alt]);
          forward(std::move(q), branches + 1, out);
        } else {
          out.push_back(std::move(p.str));
        }
        return;
      }
      const int32_t loop = p.indexOf(n1);
      if (loop >= 0) {
        noteLoop(loop);
        out.push_back(std::move(p.str));
        return;
      }
      p.push(n1, kBase[e->next]);
    }
  }

  // Assembler.pathsForward (S/Assembler.scala:236-247): longest first, ties in walk order
  std::vector<std::string> pathsForward(const std::string& start) {
    Key k{{0, 0, 0, 0}};
    bool ok = true;
    for (int j = 0; j < K; j++) {
      const int nb = nibOf(start[j]);
      if (nb < 0) { ok = false; break; }
      k.w[j >> 4] |= (uint64_t)nb << (60 - 4 * (j & 15));
    }
    if (!ok) return {start};  // a K-mer no read holds: not in the graph
    Path p;
    p.push(k, 0);
    p.str = start;
    std::vector<std::string> paths;
    forward(std::move(p), 0, paths);
    std::stable_sort(paths.begin(), paths.end(),
                     [](const std::string& a, const std::string& b) { return a.size() > b.size(); });
    return paths;
  }

  // Assembler.tryForward (S/Assembler.scala:254-267), its recursion unrolled:
  // the anchor loses K bases each time until a path extends past it by more
  // than minExtend, and the skipped bases are put back in front of every path.
  std::vector<std::string> tryForward(const std::string& anchor) {
    size_t off = 0;
    while (anchor.size() - off >= (size_t)K) {
      std::vector<std::string> paths = pathsForward(anchor.substr(off, K));
      if (!paths.empty() && paths[0].size() > anchor.size() - off + 20) {
        for (auto& p : paths) p.insert(0, anchor, 0, off);
        return paths;
      }
      off += K;
    }
    return {anchor};
  }
};

std::string revComp(const std::string& s) {  // Bases.reverseComplement: A<->T, C<->G, others kept
  std::string r(s.rbegin(), s.rend());
  for (auto& c : r) c = c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : c == 'T' ? 'A' : c;
  return r;
}

inline char up(char c) { return (c >= 'a' && c <= 'z') ? (char)(c - 32) : c; }

struct RangeError {};  // where the reference's require(...) on a region locus fails

struct Region {
  const pg_reassembly& j;
  int32_t size() const { return j.region_stop + 1 - j.region_start; }
  bool in(int32_t l) const { return l >= j.region_start && l <= j.region_stop; }
  char baseAt(int32_t l) const {
    if (!in(l)) throw RangeError();
    return up(j.bases[l - j.region_start]);
  }
  char originalBaseAt(int32_t l) const {
    if (!in(l)) throw RangeError();
    return up(j.orig[l - j.region_start]);
  }
  std::string sub(const char* b, int32_t l, int32_t n) const {  // subString / refSubString
    if (!(in(l) && in(l + n - 1))) throw RangeError();
    std::string s((size_t)std::max(n, 0), ' ');
    for (int32_t k = 0; k < n; k++) s[k] = up(b[l - j.region_start + k]);
    return s;
  }
};

struct Solution {
  int32_t start = 0;
  std::string was, patch;
  bool operator==(const Solution& o) const { return start == o.start && was == o.was && patch == o.patch; }
  size_t total() const { return was.size() + patch.size(); }
};

// GapFiller.properOverlap (S/GapFiller.scala:220-245): the first overlap, from
// minOverlap up, at which the end of `left` equals the start of `right`.
std::string properOverlap(const std::string& left, const std::string& right, int32_t minOverlap) {
  const int32_t ll = (int32_t)left.size(), rl = (int32_t)right.size();
  for (int32_t ov = minOverlap; ov <= ll + rl - 2 * minOverlap; ov++) {
    const int32_t lo = std::max(ll - ov, 0), ro = std::max(ov - ll, 0);
    const int32_t len = std::min(ll - lo, rl - ro);
    if (len <= 0 || memcmp(left.data() + lo, right.data() + ro, (size_t)len) == 0)
      return left.substr(0, (size_t)lo) + right.substr((size_t)ro);
  }
  return "";
}

// GapFiller.trimPatch (S/GapFiller.scala:247-262): drops the patch's ends that
// equal the region's bases (fixed or original) there.
Solution trimPatch(const Region& R, int32_t start, const std::string& patchIn, int32_t stop) {
  size_t a = 0, b = patchIn.size();
  while (start < stop && a < b && (R.baseAt(start) == patchIn[a] || R.originalBaseAt(start) == patchIn[a])) {
    start++;
    a++;
  }
  while (start < stop && a < b &&
         (R.baseAt(stop - 1) == patchIn[b - 1] || R.originalBaseAt(stop - 1) == patchIn[b - 1])) {
    stop--;
    b--;
  }
  Solution s;
  s.start = start;
  s.was = R.sub(R.j.orig, start, stop - start);
  s.patch = patchIn.substr(a, b - a);
  return s;
}

std::string consensusLeft(const std::vector<std::string>& s) {  // consensusFromLeft (:102-110)
  if (s.size() == 1) return s[0];
  size_t m = s[0].size();
  for (auto& x : s) m = std::min(m, x.size());
  for (size_t i = 0; i < m; i++)
    for (size_t k = 1; k < s.size(); k++)
      if (s[k][i] != s[0][i]) return s[0].substr(0, i);
  return s[0].substr(0, m);
}
std::string consensusRight(const std::vector<std::string>& s) {  // consensusFromRight (:112-123)
  if (s.size() == 1) return s[0];
  size_t m = s[0].size();
  for (auto& x : s) m = std::min(m, x.size());
  for (size_t i = 0; i < m; i++)
    for (size_t k = 1; k < s.size(); k++)
      if (s[k][s[k].size() - 1 - i] != s[0][s[0].size() - 1 - i]) return s[0].substr(s[0].size() - i);
  return s[0].substr(s[0].size() - m);
}

// GapFiller.assembleAcrossBreak (S/GapFiller.scala:49-100) on one window's graph.
Solution reassemble(const Graph& G, const pg_reassembly& job, int32_t& loopLen) {
  const Region R{job};
  const int32_t bs = job.break_start, be = job.break_stop;
  const int32_t start = std::max(bs - job.break_radius, job.region_start);
  const int32_t stop = std::min(be + 1 + job.break_radius, job.region_stop);
  const std::string left = R.sub(job.bases, start, bs - start);
  const std::string right = R.sub(job.bases, be + 1, stop - be - 1);
  Walker w{G, G.K};
  const std::vector<std::string> fromLeft = w.tryForward(left);      // Assembler.multiBridge
  std::vector<std::string> fromRight = w.tryForward(revComp(right));
  for (auto& p : fromRight) p = revComp(p);
  loopLen = w.loopLength;
  // breakJoins (:161-184): the distinct joins, a Scala Set (insertion order up
  // to four elements), sorted by total length; one change of length wins
  std::vector<Solution> set;
  const int32_t k = 2 * G.K + 1;  // GapFiller.k
  for (auto& f : fromLeft)
    for (auto& r : fromRight) {
      const std::string patch = properOverlap(f, r, k);
      if (patch.empty()) continue;
      Solution s = trimPatch(R, start, patch, stop);
      if (std::find(set.begin(), set.end(), s) == set.end()) set.push_back(std::move(s));
    }
  bool oneLength = !set.empty();
  for (auto& s : set)
    if ((int64_t)s.patch.size() - (int64_t)s.was.size() != (int64_t)set[0].patch.size() - (int64_t)set[0].was.size())
      oneLength = false;
  Solution none;
  Solution solution = none;
  if (oneLength) {
    solution = *std::min_element(set.begin(), set.end(),  // the first of the smallest, as a stable sort keeps it
                                 [](const Solution& a, const Solution& b) { return a.total() < b.total(); });
  }
  const bool isGap = job.is_gap != 0;
  bool ok = solution.start > 0 && loopLen == 0;
  if (ok && isGap) {
    const int64_t diff = (int64_t)solution.patch.size() - (int64_t)(be + 1 - bs);
    if ((diff < 0 ? -diff : diff) > job.gap_margin) ok = false;  // Pilon.gapMargin
  }
  if (ok) return solution;
  if (!(isGap || (job.fix_breaks && loopLen == 0))) return none;
  // a gap not closed (or a break, with --fix breaks): each side's consensus, with Ns between (:76-99)
  const std::string cl = consensusLeft(fromLeft), cr = consensusRight(fromRight);
  const int32_t newStart = start + (int32_t)cl.size(), newStop = stop - (int32_t)cr.size();
  bool matchesRef = false;  // partialMatchesReference (:264-281)
  if (!(start + (int32_t)cl.size() > job.region_stop || stop - (int32_t)cr.size() < job.region_start))
    matchesRef = cl == R.sub(job.bases, start, (int32_t)cl.size()) &&
                 cr == R.sub(job.bases, stop - (int32_t)cr.size(), (int32_t)cr.size());
  if ((newStart >= bs + 20 || newStop <= be - 20) && !matchesRef) {  // GapFiller.minExtend
    // Pilon.minGap; (1 to n) is empty for n <= 0
    const int32_t gapLen = isGap ? std::max(job.min_gap, newStop - newStart) : job.min_gap;
    Solution s = trimPatch(R, start, cl + std::string((size_t)std::max(gapLen, 0), 'N') + cr, stop);
    return s.patch.empty() ? none : s;
  }
  return none;
}

}  // namespace

extern "C" {

pg_status pg_scan_reads(const pg_reads* reads, const pg_params* params, int32_t n_contigs, int32_t huge,
                        int32_t threads, int64_t* stats, int64_t* strays, int64_t stray_cap, int64_t* n_first,
                        int64_t* n_second) try {
  if (!reads || !params || !stats || !n_first || !n_second || reads->n_reads < 0 || n_contigs < 0 ||
      stray_cap < 0 || (stray_cap > 0 && !strays) ||
      (reads->n_reads > 0 && (!reads->flag || !reads->tlen || !reads->l_seq || !reads->ref_id ||
                              !reads->mate_ref_id)))
    return PG_ERR_ARG;
  const int64_t n = reads->n_reads;
  const int32_t nt = (int32_t)std::max<int64_t>(1, std::min<int64_t>(
      threads > 0 ? threads : (int32_t)std::thread::hardware_concurrency(), std::max<int64_t>(1, n >> 16)));
  struct Part {
    int64_t st[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // fr, rf, unpaired: count, sum, sumSq
    std::vector<int64_t> first, second;
  };
  std::vector<Part> part((size_t)nt);
  auto work = [&](int32_t t) {
    Part& p = part[(size_t)t];
    const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    for (int64_t i = lo; i < hi; i++) {
      const uint32_t f = reads->flag[i];
      // validateRead (S/BamFile.scala:101-105), and mapped
      if ((f & 0x100) || (!params->nonpf && (f & 0x200)) || (!params->duplicates && (f & 0x400)) || (f & 0x4))
        continue;
      const bool paired = f & 0x1, proper = f & 0x2, rc = f & 0x10;
      int64_t size = -1;
      bool unpaired = false;
      if (paired && proper) size = reads->tlen[i];        // addInsert(getInferredInsertSize, reverse)
      else if (!paired) size = reads->l_seq[i], unpaired = true;  // addInsert(getReadLength, reverse, true)
      if (size > 0 && size < huge) {  // addInsert (:194-202); a kept size is positive, so FR is !reverse
        const int k = unpaired ? 6 : (rc ? 3 : 0);
        p.st[k] += 1;
        p.st[k + 1] += size;
        p.st[k + 2] += (int32_t)(uint32_t)(uint64_t)(size * size);  // size * size is a Scala Int
      }
      // strayMateMap candidates: paired, not proper, mate mapped, on a reference of interest
      if (paired && !proper && !(f & 0x8)) {
        const int32_t rid = reads->ref_id[i], mrid = reads->mate_ref_id[i];
        if ((rid >= 0 && rid < n_contigs) || (mrid >= 0 && mrid < n_contigs))
          ((f & 0x40) ? p.first : p.second).push_back(i);
      }
    }
  };
  std::vector<std::thread> pool;
  int32_t started = 1;
  try {
    pool.reserve((size_t)nt);
    for (; started < nt; started++) pool.emplace_back(work, started);
  } catch (const std::exception&) {
  }
  for (int32_t t = started; t < nt; t++) work(t);  // the shares of threads that did not start
  work(0);
  for (auto& th : pool) th.join();
  for (int k = 0; k < 9; k++) stats[k] = 0;
  int64_t nf = 0, ns = 0;
  for (const Part& p : part) {
    for (int k = 0; k < 9; k++) stats[k] += p.st[k];
    nf += (int64_t)p.first.size();
    ns += (int64_t)p.second.size();
  }
  *n_first = nf;
  *n_second = ns;
  if (nf + ns > stray_cap) return PG_ERR_LIMIT;
  int64_t o = 0;
  for (const Part& p : part)
    for (int64_t i : p.first) strays[o++] = i;
  for (const Part& p : part)
    for (int64_t i : p.second) strays[o++] = i;
  return PG_OK;
} PG_HOST_CATCH(nullptr)

pg_status pg_reassemble(const pg_kmer_edge_wide* edges, int64_t n_edges, int32_t K, const pg_reassembly* jobs,
                        int32_t n_jobs, int32_t threads, pg_reassembly_fix* fixes, char* text, int64_t text_cap,
                        int64_t* text_len) try {
  // no C++ exception crosses the C boundary: a host allocation that fails is PG_ERR_NOMEM, and
  // threads that cannot be started leave the jobs to the threads that did start
  if ((n_edges > 0 && !edges) || n_edges < 0 || n_jobs < 0 || (n_jobs > 0 && (!jobs || !fixes)) || !text_len ||
      text_cap < 0 || (text_cap > 0 && !text) || K < 1 || K > 63)
    return PG_ERR_ARG;
  int32_t n_windows = 0;
  for (int32_t i = 0; i < n_jobs; i++) {
    const pg_reassembly& j = jobs[i];
    if (j.window < 0 || !j.bases || !j.orig || j.region_start < 1 || j.region_stop < j.region_start ||
        j.break_start > j.break_stop || j.break_radius < 0)
      return PG_ERR_ARG;
    n_windows = std::max(n_windows, j.window + 1);
  }
  for (int64_t e = 0; e < n_edges; e++)
    if (edges[e].window < 0) return PG_ERR_ARG;
  // each window's edges, grouped by a counting sort
  std::vector<int64_t> start((size_t)n_windows + 1, 0), order;
  for (int64_t e = 0; e < n_edges; e++)
    if (edges[e].window < n_windows) start[edges[e].window + 1]++;
  for (int32_t w = 0; w < n_windows; w++) start[w + 1] += start[w];
  order.resize((size_t)start[n_windows]);
  {
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int64_t e = 0; e < n_edges; e++)
      if (edges[e].window < n_windows) order[fill[edges[e].window]++] = e;
  }
  std::vector<Solution> sol((size_t)n_jobs);
  std::vector<int32_t> status((size_t)n_jobs, PG_OK), loops((size_t)n_jobs, 0);
  std::atomic<int32_t> next{0};
  auto work = [&]() {
    for (int32_t i; (i = next.fetch_add(1)) < n_jobs;) {
      const pg_reassembly& j = jobs[i];
      const int64_t e0 = start[j.window], e1 = start[j.window + 1];
      try {
        Graph G(K, (size_t)(e1 - e0));
        for (int64_t t = e0; t < e1; t++) {
          const pg_kmer_edge_wide& e = edges[order[t]];
          Edge* v = G.g.insert(Key{{e.key[0], e.key[1], e.key[2], e.key[3]}});
          v->next = e.next;
          v->alt = e.alt;
        }
        sol[i] = reassemble(G, j, loops[i]);
      } catch (RangeError&) {
        status[i] = PG_ERR_INDEX;
      } catch (...) {
        sol[i] = Solution();
        status[i] = pg::host_exception_status(nullptr);
      }
    }
  };
  const int32_t nt = std::max(1, std::min(threads > 0 ? threads : (int32_t)std::thread::hardware_concurrency(), n_jobs));
  std::vector<std::thread> pool;
  pool.reserve((size_t)nt);
  for (int32_t t = 1; t < nt; t++) {
    try {
      pool.emplace_back(work);
    } catch (const std::exception&) {
      break;
    }
  }
  work();
  for (auto& t : pool) t.join();
  int64_t off = 0;
  pg_status rc = PG_OK;
  for (int32_t i = 0; i < n_jobs; i++) {
    pg_reassembly_fix& f = fixes[i];
    f.start = status[i] == PG_OK ? sol[i].start : 0;
    f.status = status[i];
    f.loop_len = loops[i];
    f.pad_ = 0;
    f.was_off = off;
    f.was_len = (int64_t)sol[i].was.size();
    if (off + f.was_len <= text_cap) memcpy(text + off, sol[i].was.data(), sol[i].was.size());
    off += f.was_len;
    f.patch_off = off;
    f.patch_len = (int64_t)sol[i].patch.size();
    if (off + f.patch_len <= text_cap) memcpy(text + off, sol[i].patch.data(), sol[i].patch.size());
    off += f.patch_len;
  }
  *text_len = off;
  if (off > text_cap) rc = PG_ERR_LIMIT;
  for (int32_t i = 0; i < n_jobs; i++)
    if (status[i] == PG_ERR_NOMEM || status[i] == PG_ERR_LIMIT) rc = (pg_status)status[i];
  return rc;
} PG_HOST_CATCH(nullptr)

}  // extern "C"
