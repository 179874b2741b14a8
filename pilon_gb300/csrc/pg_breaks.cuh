// pg_breaks.cuh — arguments of the break-candidate kernels (pg_breaks.cu).
#pragma once
#include "pg_internal.cuh"

namespace pg {

constexpr int kBreakStarts = 12;  // run starts inside one 1024-position tile (slop 100: at most 10)

struct BreakTile {                // per call tile; test 0 = break, test 1 = reference N
  int32_t first[2], last[2], n[2];
  int32_t start[2][kBreakStarts], prev[2][kBreakStarts];
};

struct BreakArgs {
  const RegionDev* regions;
  const int32_t* call_tile_region;
  int32_t tile_begin, n_tiles;
  Records rec;
  const StatsDev* stats;
  const uint8_t* ref;
  int32_t min_min_depth;
  int32_t* frag;                  // per position: fragCoverage
  long long* sums;                // per region: fragCoverage, badCoverage, coverage sums
  BreakTile* tiles;
  int2* gap_scratch;              // per call tile kBreakStarts + 1 gap runs
  int2* brk_scratch;              // per call tile kBreakStarts + 1 break runs
  int32_t* brk_count;             // per region, then the exclusive scan (n_regions + 1)
  int32_t* brk_off;
  pg_break* out;                  // all breaks, by region then position
};

void launch_breaks(const BreakArgs& a, int32_t n_regions, cudaStream_t s);
// GenomeRegion.duplicationEvents of every region from the fragCoverage and sums
// that launch_breaks computed: tile_runs holds one int2 per call tile; the
// duplications go to out (unordered) and their number to *n_out.
void launch_duplications(const BreakArgs& a, int32_t n_regions, int2* tile_runs, pg_break* out, int64_t cap,
                         unsigned long long* n_out, cudaStream_t s);
// Windows of the K-mer tally from the breaks: the reads of the break's contig
// that start in [start - radius - max_span, stop + radius] (the read store's
// index, like the host's ReadIndex.range_for).
void launch_break_windows(const Reads& R, const RegionDev* regions, const pg_break* brk, int32_t n,
                          int32_t radius, const ReadExtent* ext, pg_window* out, cudaStream_t s);

}  // namespace pg
