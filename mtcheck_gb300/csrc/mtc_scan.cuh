// mtc_scan.cuh -- deterministic block/grid scans used by the compaction,
// gather and restart kernels.  Results never depend on scheduling order.
#pragma once
#include <cstdlib>
#include <cstdint>
#include <cuda_runtime.h>

#include "mtc_internal.hpp"

namespace mtc {

constexpr int kScanThreads = 512;
constexpr int kScanPerThread = 8;
constexpr int kScanTile = kScanThreads * kScanPerThread;  // 4096 elements per tile

__device__ __forceinline__ uint64_t warp_incl_scan(uint64_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Exclusive scan of one value per thread across the block (blockDim.x <= 1024,
// multiple of 32).  `total` receives the block sum.  Uses `sh` (>= 32 slots).
__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, uint64_t* sh, uint64_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint64_t incl = warp_incl_scan(v);
  if (lane == 31) sh[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint64_t w = lane < nw ? sh[lane] : 0;
    uint64_t wi = warp_incl_scan(w);
    if (lane < nw) sh[lane] = wi - w;
    if (lane == nw - 1) sh[32] = wi;
  }
  __syncthreads();
  uint64_t r = incl - v + sh[warp];
  if (total) *total = sh[32];
  __syncthreads();
  return r;
}

// Grid-level exclusive scan of u64 values produced by a functor, three phases.
//   phase 1: tile sums         (grid over tiles)
//   phase 2: scan of tile sums (one block)
//   phase 3: per-element exclusive prefix, consumer functor called with it
// `n` is read from device memory so that launches do not depend on host-known
// counts (the grid covers `max_n`).
template <class Val>
__global__ void scan_tile_sums_kernel(Val val, const uint32_t* n_ptr, uint64_t n_const, uint64_t* tile_sums) {
  pdl_enter();
  __shared__ uint64_t sh[33];
  const uint64_t n = n_ptr ? *n_ptr : n_const;
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  uint64_t s = 0;
  if (base < n) {
    for (int k = 0; k < kScanPerThread; k++) {
      uint64_t i = base + (uint64_t)k * kScanThreads + threadIdx.x;
      if (i < n) s += val(i);
    }
  }
  uint64_t total;
  block_excl_scan(s, sh, &total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// single block: exclusive scan of tile sums in place; grand total to *total
static __global__ void scan_tile_offsets_kernel(uint64_t* tile_sums, uint32_t ntiles, uint64_t* total) {
  pdl_enter();
  __shared__ uint64_t sh[33];
  uint64_t carry = 0;
  for (uint32_t b = 0; b < ntiles; b += blockDim.x) {
    uint32_t i = b + threadIdx.x;
    uint64_t v = i < ntiles ? tile_sums[i] : 0;
    uint64_t t;
    uint64_t ex = block_excl_scan(v, sh, &t);
    if (i < ntiles) tile_sums[i] = carry + ex;
    carry += t;
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

// Each element i gets (offset of its tile) + exclusive prefix inside the tile;
// elements are visited in ascending order per thread chunk so that the
// consumer sees a stable order.
template <class Val, class Emit>
__global__ void scan_emit_kernel(Val val, Emit emit, const uint32_t* n_ptr, uint64_t n_const, const uint64_t* tile_offsets) {
  pdl_enter();
  __shared__ uint64_t sh[33];
  const uint64_t n = n_ptr ? *n_ptr : n_const;
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  if (base >= n) return;
  // thread t owns the contiguous run [base + t*PER, base + (t+1)*PER)
  uint64_t v[kScanPerThread];
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanPerThread; k++) {
    uint64_t i = base + (uint64_t)threadIdx.x * kScanPerThread + k;
    v[k] = i < n ? val(i) : 0;
    s += v[k];
  }
  uint64_t ex = block_excl_scan(s, sh, nullptr) + tile_offsets[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanPerThread; k++) {
    uint64_t i = base + (uint64_t)threadIdx.x * kScanPerThread + k;
    if (i < n) emit(i, ex, v[k]);
    ex += v[k];
  }
}

// Phases 2 and 3 in one launch, for grids of at most kReduceTiles tiles: each
// block sums the sums of the tiles before it; the block holding element n-1
// (block 0 when n is 0) writes the grand total.
constexpr uint32_t kReduceTiles = 2048;
// The largest grid the two-launch forms serve: kReduceTiles, or less under the
// test hook MTCHECK_REDUCE_TILES, which sends small inputs down the
// three-launch path that otherwise only inputs of more than 2^23 elements take.
inline uint32_t reduce_tile_limit() {
  const char* e = std::getenv("MTCHECK_REDUCE_TILES");
  if (e && *e) {
    const unsigned long v = std::strtoul(e, nullptr, 10);
    if (v < kReduceTiles) return (uint32_t)v;
  }
  return kReduceTiles;
}
template <class Val, class Emit>
__global__ void scan_emit_reduce_kernel(Val val, Emit emit, const uint32_t* n_ptr, uint64_t n_const,
                                        const uint64_t* tile_sums, uint64_t* total) {
  pdl_enter();
  __shared__ uint64_t sh[33];
  const uint64_t n = n_ptr ? *n_ptr : n_const;
  const uint64_t last_tile = n ? (n - 1) / kScanTile : 0;
  if (blockIdx.x > last_tile) return;
  uint64_t part = 0;
  for (uint32_t k = threadIdx.x; k < blockIdx.x; k += blockDim.x) part += tile_sums[k];
  uint64_t off;
  block_excl_scan(part, sh, &off);
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile;
  uint64_t v[kScanPerThread];
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanPerThread; k++) {
    uint64_t i = base + (uint64_t)threadIdx.x * kScanPerThread + k;
    v[k] = i < n ? val(i) : 0;
    s += v[k];
  }
  uint64_t tile_total;
  uint64_t ex = block_excl_scan(s, sh, &tile_total) + off;
  if (total && blockIdx.x == last_tile && threadIdx.x == 0) *total = off + tile_total;
#pragma unroll
  for (int k = 0; k < kScanPerThread; k++) {
    uint64_t i = base + (uint64_t)threadIdx.x * kScanPerThread + k;
    if (i < n) emit(i, ex, v[k]);
    ex += v[k];
  }
}

// Host helper: run the three phases (two launches up to kReduceTiles tiles).  `scratch` holds >= ceil(max_n/kScanTile)+1
// u64; `total` (device) receives the grand total.
template <class Val, class Emit>
inline cudaError_t grid_scan(Val val, Emit emit, const uint32_t* n_dev, uint64_t max_n, uint64_t* scratch,
                             uint64_t* total, cudaStream_t s) {
  uint32_t ntiles = (uint32_t)((max_n + kScanTile - 1) / kScanTile);
  if (ntiles == 0) ntiles = 1;
  launch_k(scan_tile_sums_kernel<Val>, ntiles, kScanThreads, 0, s, val, n_dev, max_n, scratch);
  if (ntiles <= reduce_tile_limit()) {
    launch_k(scan_emit_reduce_kernel<Val, Emit>, ntiles, kScanThreads, 0, s, val, emit, n_dev, max_n,
             (const uint64_t*)scratch, total);
    note_launch(2);
    return cudaGetLastError();
  }
  launch_k(scan_tile_offsets_kernel, 1, 1024, 0, s, scratch, ntiles, total);
  launch_k(scan_emit_kernel<Val, Emit>, ntiles, kScanThreads, 0, s, val, emit, n_dev, max_n,
           (const uint64_t*)scratch);
  note_launch(3);
  return cudaGetLastError();
}

}  // namespace mtc
