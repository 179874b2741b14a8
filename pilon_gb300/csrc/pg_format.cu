// pg_format.cu — VCF text for one region, formatted on the device.
//
// Vcf.writeRecord (S/Vcf.scala:74-176) writes one record per position plus a
// second record after indel calls.  Here every position's records are
// formatted by one thread in two passes: the first only measures the bytes,
// an exclusive scan turns the lengths into offsets, and the second writes the
// text at its offset.  The host writes the header, any <DUP> records and the
// buffer.
//
// AF is "%.2f" of (float)altDP / (float)(refDP + altDP) widened to double.
// Java's Formatter rounds HALF_UP on the shortest decimal digits of that
// double.  For a float-valued double f, 100 * f is exact in double (24 + 7 <
// 53 mantissa bits), and f can only sit exactly on a two-decimal tie when it
// is a multiple of 1/8; there the shortest digits are the tie itself, so
// Java's rule equals rounding 100 * f half up.  That is what fmt_af does.
#include <cuda_runtime.h>

#include <algorithm>

#include "pg_format.cuh"
#include "pg_internal.cuh"

namespace pg {

struct Out {  // measuring (buf == nullptr) or writing writer
  char* buf;
  int64_t n;
  __device__ inline void c(char ch) {
    if (buf) buf[n] = ch;
    n++;
  }
  __device__ inline void s(const char* p) {
    while (*p) c(*p++);
  }
  __device__ inline void bytes(const uint8_t* p, int32_t len) {
    for (int32_t k = 0; k < len; k++) c((char)p[k]);
  }
  __device__ inline void i64(int64_t v) {
    char t[24];
    int k = 0;
    uint64_t u = v < 0 ? (uint64_t)(-(v + 1)) + 1 : (uint64_t)v;
    do {
      t[k++] = (char)('0' + (int)(u % 10));
      u /= 10;
    } while (u);
    if (v < 0) c('-');
    while (k) c(t[--k]);
  }
};

__device__ inline void fmt_af(Out& o, int32_t alt, int32_t tot) {
  // tot > 0 here; the float ratio as Java computes it, widened to double
  const float f = (float)alt / (float)tot;
  const double d = (double)f * 100.0;  // exact
  double fl = floor(d);
  if (d - fl >= 0.5) fl += 1.0;        // HALF_UP (ties only at multiples of 1/8)
  const int64_t v = (int64_t)fl;       // hundredths
  if (v < 0) {
    o.c('-');
    o.i64(-v / 100);
  } else {
    o.i64(v / 100);
  }
  const int64_t r = v < 0 ? (-v) % 100 : v % 100;
  o.c('.');
  o.c((char)('0' + r / 10));
  o.c((char)('0' + r % 10));
}

struct PosView {
  int64_t cnt[4], qs[4];
  int32_t mq_sum, q_sum, phys_cov, bad_pair, deletions, del_qual, insertions, ins_qual, clips;
  uint32_t call;
  int64_t score;
  int32_t indel_len, ins_str;
};

// One writeRecord call.  `lead`: reference base before the locus (indel records).
__device__ void vcf_record(Out& o, const FormatArgs& A, const PosView& v, int32_t index, bool embedded,
                           bool indelOkArg) {
  const RegionDev& g = A.region;
  const bool indelOk = indelOkArg && index > 0;
  const int32_t locus = g.start + index;
  const uint32_t f = v.call;
  const int64_t n = v.cnt[0] + v.cnt[1] + v.cnt[2] + v.cnt[3];
  const int64_t depthL = n + v.deletions;
  const int b = (int)(f & 3u), ab = (int)((f >> 2) & 3u);
  const char base = (f & PG_CALL_HAS_BASE) ? "ACGT"[b] : 'N';
  const char altBase = "ACGT"[ab];
  const bool homo = f & PG_CALL_HOMO, isIns = f & PG_CALL_INS, isDel = f & PG_CALL_DEL;
  const bool homoIndel = f & PG_CALL_HOMO_INDEL;
  const int64_t baseSum = pick4(v.qs, b), altBaseSum = pick4(v.qs, ab);
  const int32_t baseDP = (int32_t)baseSum, altBaseDP = (int32_t)altBaseSum;
  const int32_t depth = (int32_t)depthL;
  const uint8_t* cref = A.ref + g.ref_off;
  auto refBase = [&](int32_t l) -> char { return (char)upper(cref[l - 1]); };
  // callString(indelOk): the insertion, the deletion or the base
  const bool csIns = indelOk && isIns, csDel = !csIns && indelOk && isDel;
  const uint8_t* ins = (isIns && v.ins_str >= 0) ? (const uint8_t*)A.pool + v.ins_str : nullptr;
  const uint8_t* del = cref + (locus - 1);  // deletion string: reference bytes [locus-1, locus-1+len)
  int32_t loc = locus;
  // rBase / cBase as (first char, optional tail)
  char r0, c0;
  const uint8_t* rt = nullptr;
  int32_t rtl = 0;
  const uint8_t* ct = nullptr;
  int32_t ctl = 0;
  int callType;             // 0 "0/0", 1 "0/1", 2 "1/1"
  int32_t refDP, altDP;
  if (indelOk && !embedded && isDel) {
    loc -= 1;
    const char rb = refBase(loc);
    callType = homoIndel ? 2 : 1;
    const int32_t p = max(pctI(v.del_qual, v.mq_sum), pctI(v.deletions, wadd((int32_t)n, v.deletions)));
    r0 = rb; rt = del; rtl = v.indel_len;
    c0 = rb;
    refDP = 100 - p; altDP = p;
  } else if (indelOk && !embedded && isIns) {
    loc -= 1;
    const char rb = refBase(loc);
    callType = homoIndel ? 2 : 1;
    const int32_t p = max(pctI(v.ins_qual, v.mq_sum), pctI(v.insertions, (int32_t)n));
    r0 = rb;
    c0 = rb; ct = ins; ctl = v.indel_len;
    refDP = 100 - p; altDP = p;
  } else if (homo) {
    const char rb = refBase(loc);
    r0 = rb;
    c0 = base;
    const bool bcIsN = !csIns && !csDel && base == 'N';
    if (rb == base || bcIsN) { callType = 0; refDP = baseDP; altDP = altBaseDP; }
    else { callType = 2; refDP = altBaseDP; altDP = baseDP; }
  } else {
    const char rb = refBase(loc);
    r0 = rb;
    if (rb == base) { c0 = altBase; callType = 1; refDP = baseDP; altDP = altBaseDP; }
    else { c0 = base; callType = 1; refDP = altBaseDP; altDP = baseDP; }
  }
  // cBaseVcf: "." when cBase is "N" or equals rBase
  const int32_t rlen = 1 + rtl, clen = 1 + ctl;
  bool dot = false;
  if (clen == 1 && c0 == 'N') dot = true;
  if (clen == 1 && rlen == 1 && c0 == r0) dot = true;
  if (A.variants_only && dot) return;  // deltas: only records with an alternate allele
  // line
  o.bytes((const uint8_t*)A.name, A.name_len);
  o.c('\t');
  o.i64(loc);
  o.s("\t.\t");
  o.c(r0);
  if (rtl) o.bytes(rt, rtl);
  o.c('\t');
  if (dot) o.c('.');
  else {
    o.c(c0);
    if (ctl) o.bytes(ct, ctl);
  }
  o.c('\t');
  if (indelOk && isDel) o.c('.');
  else o.i64(v.score);
  o.c('\t');
  // filters are prepended in the reference: Del;Amb;LowCov order
  bool any = false;
  if (embedded) { o.s("Del"); any = true; }
  if (!A.diploid && callType == 1) { if (any) o.c(';'); o.s("Amb"); any = true; }
  if (depth < A.min_depth) { if (any) o.c(';'); o.s("LowCov"); any = true; }
  if (!any) o.s("PASS");
  o.s("\tDP=");
  o.i64(!embedded ? depthL : n);
  o.s(";TD=");
  o.i64(depthL + v.bad_pair);
  o.s(";BQ=");
  const int64_t tqs = v.qs[0] + v.qs[1] + v.qs[2] + v.qs[3];
  o.i64(roundDivL(tqs, roundDivL((int64_t)v.mq_sum * n, depthL)));
  o.s(";MQ=");
  o.i64(roundDivL((int64_t)v.mq_sum - depthL, depthL));
  o.s(";QD=");
  o.i64(n > 0 ? v.score / n : 0);
  o.s(";BC=");
  for (int k = 0; k < 4; k++) { if (k) o.c(','); o.i64(v.cnt[k]); }
  if (A.vcf_qe) {
    o.s(";QE=");
    for (int k = 0; k < 4; k++) { if (k) o.c(','); o.i64(v.qs[k]); }
  } else {
    o.s(";QP=");
    for (int k = 0; k < 4; k++) {
      if (k) o.c(',');
      o.i64(tqs == 0 ? 0 : (100 * v.qs[k] + tqs / 2) / tqs);
    }
  }
  o.s(";PC=");
  o.i64(v.phys_cov);
  o.s(";IC=");
  o.i64(v.insertions);
  o.s(";DC=");
  o.i64(v.deletions);
  o.s(";XC=");
  o.i64(v.clips);
  o.s(";AC=");
  o.c((char)('0' + callType));
  o.s(";AF=");
  const int32_t tot = wadd(refDP, altDP);
  if (tot > 0 && !dot) fmt_af(o, altDP, tot);
  else o.s("0.00");
  o.s("\tGT\t");
  o.s(callType == 0 ? "0/0" : callType == 1 ? "0/1" : "1/1");
  o.c('\n');
}

__device__ inline void load_view(const FormatArgs& A, int64_t gp, PosView& v) {
  const Records& R = A.rec;
  const int4 c = R.count[gp];
  v.cnt[0] = c.x; v.cnt[1] = c.y; v.cnt[2] = c.z; v.cnt[3] = c.w;
  const longlong2 a = R.qual_sum[2 * gp], b = R.qual_sum[2 * gp + 1];
  v.qs[0] = a.x; v.qs[1] = a.y; v.qs[2] = b.x; v.qs[3] = b.y;
  v.mq_sum = R.mq_sum[gp]; v.q_sum = R.q_sum[gp]; v.phys_cov = R.phys_cov[gp]; v.bad_pair = R.bad_pair[gp];
  v.deletions = R.deletions[gp]; v.del_qual = R.del_qual[gp]; v.insertions = R.insertions[gp];
  v.ins_qual = R.ins_qual[gp]; v.clips = R.clips[gp]; v.call = R.call[gp]; v.score = R.score[gp];
  v.indel_len = R.indel_len[gp]; v.ins_str = R.ins_str[gp];
}

// GenomeRegion.writeVcf's per-position part (S/GenomeRegion.scala:623-643)
__device__ inline int64_t vcf_position(const FormatArgs& A, int32_t i, char* buf) {
  PosView v;
  load_view(A, A.region.pos_base + i, v);
  const bool deleted = v.call & PG_CALL_DELETED;
  Out o{buf, 0};
  vcf_record(o, A, v, i, deleted, true);
  const bool indel = v.call & (PG_CALL_INS | PG_CALL_DEL);
  if (i > 0 && indel && !deleted) {
    const bool emb = (v.call & PG_CALL_DEL) && (v.call & PG_CALL_HOMO_INDEL);
    vcf_record(o, A, v, i, emb, false);
  }
  return o.n;
}

__global__ void k_vcf_len(FormatArgs A, int64_t* len) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.region.size) return;
  len[i] = vcf_position(A, i, nullptr);
}

__global__ void k_vcf_write(FormatArgs A, const int64_t* off, char* text) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.region.size) return;
  vcf_position(A, i, text + off[i]);
}

// exclusive scan of int64 lengths: per-1024 block sums, one CTA over the sums, apply
__device__ inline int64_t block_excl_scan(int64_t v, int64_t* s_w, int64_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    int64_t w = lane < nw ? s_w[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    s_w[lane] = w;
  }
  __syncthreads();
  const int64_t incl = x + (warp > 0 ? s_w[warp - 1] : 0);
  total = s_w[(blockDim.x >> 5) - 1];
  __syncthreads();
  return incl - v;
}

__global__ void __launch_bounds__(1024) k_scan64_a(const int64_t* in, int64_t n, int64_t* sums) {
  __shared__ int64_t s_w[32];
  const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  int64_t tot;
  block_excl_scan(i < n ? in[i] : 0, s_w, tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan64_b(int64_t* sums, int32_t nb) {
  __shared__ int64_t s_w[32];
  __shared__ int64_t s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int32_t base = 0; base < nb; base += 1024) {
    const int32_t i = base + threadIdx.x;
    int64_t tot;
    const int64_t e = block_excl_scan(i < nb ? sums[i] : 0, s_w, tot);
    const int64_t c = s_carry;
    if (i < nb) sums[i] = c + e;
    __syncthreads();
    if (threadIdx.x == 0) s_carry = c + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[nb] = s_carry;
}

__global__ void __launch_bounds__(1024) k_scan64_c(int64_t* io, int64_t n, const int64_t* sums) {
  __shared__ int64_t s_w[32];
  const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  int64_t tot;
  const int64_t e = block_excl_scan(i < n ? io[i] : 0, s_w, tot);
  if (i < n) io[i] = e + sums[blockIdx.x];
}

void launch_vcf_lengths(const FormatArgs& A, int64_t* len, cudaStream_t s) {
  const int32_t n = A.region.size;
  if (n <= 0) return;
  k_vcf_len<<<(n + 255) / 256, 256, 0, s>>>(A, len);
}

void launch_scan64(int64_t* io, int64_t n, int64_t* sums, cudaStream_t s) {
  if (n <= 0) return;
  const int32_t nb = (int32_t)((n + 1023) / 1024);
  k_scan64_a<<<nb, 1024, 0, s>>>(io, n, sums);
  k_scan64_b<<<1, 1024, 0, s>>>(sums, nb);
  k_scan64_c<<<nb, 1024, 0, s>>>(io, n, sums);
}

__global__ void k_mark_deleted(uint32_t* call, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) call[i] |= PG_CALL_DELETED;
}

void launch_mark_deleted(uint32_t* call, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  k_mark_deleted<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(call, n);
}

void launch_vcf_write(const FormatArgs& A, const int64_t* off, char* text, cudaStream_t s) {
  const int32_t n = A.region.size;
  if (n <= 0) return;
  k_vcf_write<<<(n + 255) / 256, 256, 0, s>>>(A, off, text);
}

}  // namespace pg
