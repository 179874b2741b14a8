// pg_noalloc.cu — pg_phys_cov_scan_static: the physical-coverage prefix scan of
// one region for callers that cannot allocate device memory.
//
// Who needs it: a host that owns the whole device memory budget through its
// own pool (a JVM host with a pooled allocator, a process whose PyTorch
// caching allocator already holds the free memory) cannot let a library call
// cudaMalloc: the call may fail or fragment the pool, and it synchronises the
// device.  This entry point takes the caller's device buffers for input and
// output and keeps its only scratch, the per-tile partial sums, in a fixed
// file-scope device array.
//
// Limits and sharing: the array holds kStaticMaxTiles tiles of 1024 positions
// (16,777,216 positions, enough for a 10 Mb Pilon region), 128 KiB that every
// GPU which loads this library keeps until the process exits.  All calls share
// it and it keeps the previous call's partial sums; every tile slot a call
// reads is first written by that same call, so nothing has to be cleared.
// Calls whose kernels overlap on the GPU (different streams, or different host
// threads on one device) race on the array and must be serialised by the
// caller.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "pilon_gb300.h"

namespace {

constexpr int kTile = 1024;
constexpr int kStaticMaxTiles = 16384;
static_assert((long long)kTile * kStaticMaxTiles == PG_STATIC_SCAN_MAX_POSITIONS, "header limit");

// Scratch: two int32 partial sums (physical coverage, insert size) per tile.
static __device__ __align__(256) int32_t g_scan_scratch[2 * kStaticMaxTiles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
int32_t* g_scratch_ptr[kMaxDevices] = {nullptr};

__device__ inline void scan_pair(uint32_t& a, uint32_t& b, uint32_t* s_a, uint32_t* s_b) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t ya = __shfl_up_sync(0xffffffffu, a, o), yb = __shfl_up_sync(0xffffffffu, b, o);
    if (lane >= o) { a += ya; b += yb; }
  }
  if (lane == 31) { s_a[warp] = a; s_b[warp] = b; }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t wa = lane < nw ? s_a[lane] : 0u, wb = lane < nw ? s_b[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t ya = __shfl_up_sync(0xffffffffu, wa, o), yb = __shfl_up_sync(0xffffffffu, wb, o);
      if (lane >= o) { wa += ya; wb += yb; }
    }
    s_a[lane] = wa; s_b[lane] = wb;
  }
  __syncthreads();
  if (warp > 0) { a += s_a[warp - 1]; b += s_b[warp - 1]; }
}

// Phase 1: per-tile sums of the two difference arrays into the scratch.
__global__ void __launch_bounds__(kTile) k_static_tile_sums(const int32_t* pd, const int32_t* id, int64_t n,
                                                             int32_t* scratch) {
  __shared__ uint32_t s_a[32], s_b[32];
  const int64_t p = (int64_t)blockIdx.x * kTile + threadIdx.x;
  uint32_t a = p < n ? (uint32_t)pd[p] : 0u, b = p < n ? (uint32_t)id[p] : 0u;
  scan_pair(a, b, s_a, s_b);
  if (threadIdx.x == kTile - 1) { scratch[2 * blockIdx.x] = (int32_t)a; scratch[2 * blockIdx.x + 1] = (int32_t)b; }
}

// Phase 2: exclusive scan of the tile sums, seeded with the region's carry
// (physCovStart / insertSizeStart), in one CTA.
__global__ void __launch_bounds__(kTile) k_static_tile_scan(int32_t n_tiles, int32_t phys_start, int32_t ins_start,
                                                             int32_t* scratch) {
  __shared__ uint32_t s_a[32], s_b[32];
  __shared__ uint32_t s_ca, s_cb;
  if (threadIdx.x == 0) { s_ca = (uint32_t)phys_start; s_cb = (uint32_t)ins_start; }
  __syncthreads();
  for (int32_t base = 0; base < n_tiles; base += kTile) {
    const int32_t t = base + threadIdx.x;
    const uint32_t va = t < n_tiles ? (uint32_t)scratch[2 * t] : 0u, vb = t < n_tiles ? (uint32_t)scratch[2 * t + 1] : 0u;
    uint32_t a = va, b = vb;
    scan_pair(a, b, s_a, s_b);
    const uint32_t ca = s_ca, cb = s_cb;
    if (t < n_tiles) { scratch[2 * t] = (int32_t)(ca + a - va); scratch[2 * t + 1] = (int32_t)(cb + b - vb); }
    __syncthreads();
    if (threadIdx.x == kTile - 1) { s_ca = ca + a; s_cb = cb + b; }
    __syncthreads();
  }
}

// Phase 3: in-tile scan plus the tile's prefix; insertSize /= physCov where
// physCov > 0 (S/PileUpRegion.scala:90-100).
__global__ void __launch_bounds__(kTile) k_static_apply(const int32_t* pd, const int32_t* id, int64_t n,
                                                         const int32_t* scratch, int32_t* po, int32_t* io) {
  __shared__ uint32_t s_a[32], s_b[32];
  const int64_t p = (int64_t)blockIdx.x * kTile + threadIdx.x;
  uint32_t a = p < n ? (uint32_t)pd[p] : 0u, b = p < n ? (uint32_t)id[p] : 0u;
  scan_pair(a, b, s_a, s_b);
  if (p < n) {
    const int32_t pc = (int32_t)(a + (uint32_t)scratch[2 * blockIdx.x]);
    int32_t is = (int32_t)(b + (uint32_t)scratch[2 * blockIdx.x + 1]);
    if (pc > 0) is = is / pc;
    po[p] = pc;
    io[p] = is;
  }
}

pg_status report(char* errbuf, int32_t errcap, pg_status s, const char* msg) {
  if (errbuf && errcap > 0) snprintf(errbuf, (size_t)errcap, "%s", msg);
  return s;
}

}  // namespace

extern "C" pg_status pg_phys_cov_scan_static(const int32_t* phys_diff, const int32_t* insert_diff,
                                             int64_t n_positions, int32_t phys_cov_start,
                                             int32_t insert_size_start, int32_t* phys_cov, int32_t* insert_size,
                                             void* stream, char* errbuf, int32_t errcap) {
  if (n_positions < 0 || (n_positions > 0 && (!phys_diff || !insert_diff || !phys_cov || !insert_size)))
    return report(errbuf, errcap, PG_ERR_ARG, "null buffer or negative size");
  if (n_positions > PG_STATIC_SCAN_MAX_POSITIONS) {
    char msg[160];
    snprintf(msg, sizeof msg, "%lld positions exceed the static scratch limit of %lld positions",
             (long long)n_positions, (long long)PG_STATIC_SCAN_MAX_POSITIONS);
    return report(errbuf, errcap, PG_ERR_LIMIT, msg);
  }
  if (n_positions == 0) return PG_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return report(errbuf, errcap, PG_ERR_CUDA, "no current CUDA device");
  }
  int32_t* scratch;
  {
    // Set-up, once per device, with that device current: the device address
    // of the scratch array.  (In host code the array's name is only a host
    // stand-in.)  This first call on a device must come before any stream
    // capture that includes this entry point.  The address is kept until the
    // process exits: cudaDeviceReset (which destroys the primary context and
    // this array with it) ends the use of this entry point on that device.
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_scan_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return report(errbuf, errcap, PG_ERR_CUDA, "cudaGetSymbolAddress of the scan scratch failed");
      }
      g_scratch_ptr[dev] = (int32_t*)p;
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int32_t n_tiles = (int32_t)((n_positions + kTile - 1) / kTile);
  k_static_tile_sums<<<n_tiles, kTile, 0, s>>>(phys_diff, insert_diff, n_positions, scratch);
  k_static_tile_scan<<<1, kTile, 0, s>>>(n_tiles, phys_cov_start, insert_size_start, scratch);
  k_static_apply<<<n_tiles, kTile, 0, s>>>(phys_diff, insert_diff, n_positions, scratch, phys_cov, insert_size);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return report(errbuf, errcap, PG_ERR_CUDA, cudaGetErrorString(e));
  return PG_OK;
}
