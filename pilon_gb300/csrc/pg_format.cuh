// pg_format.cuh — arguments of the device VCF formatter (pg_format.cu).
#pragma once
#include "pg_internal.cuh"

namespace pg {

struct FormatArgs {
  RegionDev region;
  Records rec;
  const uint8_t* ref;    // concatenated reference
  const char* pool;      // insertion-call strings
  const char* name;      // contig name (device copy)
  int32_t name_len;
  int32_t min_depth;     // GenomeRegion.minDepth
  int32_t diploid;       // --diploid
  int32_t vcf_qe;        // --vcfqe
  int32_t variants_only; // skip records whose ALT is "."
};

void launch_vcf_lengths(const FormatArgs& A, int64_t* len, cudaStream_t s);
void launch_scan64(int64_t* io, int64_t n, int64_t* sums, cudaStream_t s);
void launch_vcf_write(const FormatArgs& A, const int64_t* off, char* text, cudaStream_t s);
// sets PG_CALL_DELETED on call[0, n)
void launch_mark_deleted(uint32_t* call, int64_t n, cudaStream_t s);

}  // namespace pg
