// noalloc.cu -- a checkpoint entry point that allocates no memory at all.
//
// Who needs it: code that runs where memory allocation is not allowed or not
// safe -- inside a custom allocator or an out-of-memory handler, from a
// signal or crash handler that snapshots state before the process dies, or
// inside a runtime whose memory pool owns the whole GPU.  Such callers can
// still hand over the buffers they already own.
//
// What it does: the basic approach (src/basic_approach.cpp:14-143) without a
// deduplicator object.  The caller owns the per-chunk digests of the previous
// checkpoint (updated in place) and a device output buffer that receives the
// .basic incremental checkpoint: header, ids of the changed chunks in
// ascending order, and their data.  The bytes are the same as those of a
// basic-approach deduplicator that has seen the same sequence of buffers.
//
// Scratch: one changed-flag byte per chunk plus one scan word per 4096 chunks,
// held in the file-scope device array below.  Every GPU that loads the library
// keeps this array (kNoAllocScratchBytes) for the lifetime of the process.
// All calls share it and each call rewrites everything it reads, so nothing
// has to be cleared between calls; calls that run at the same time on the GPU
// (different streams or threads) race on it and must be serialised by the
// caller.
#include <cstring>

#include "../../include/mtcheck.h"
#include "mtc_internal.hpp"
#include "mtc_scan.cuh"

namespace mtc {
namespace {

constexpr uint64_t kNoAllocMaxChunks = 1ull << 22;                    // 4 Mi chunks
constexpr uint64_t kNoAllocTiles = kNoAllocMaxChunks / kScanTile + 1;  // scan words
constexpr uint64_t kNoAllocScratchBytes = kNoAllocMaxChunks + 8 * (kNoAllocTiles + 2);

// [flags: kNoAllocMaxChunks bytes][tile sums: kNoAllocTiles u64][total: 1 u64][spare]
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocArgs {
  const uint8_t* data;
  uint64_t len;
  uint32_t cs, n;
  const uint8_t* flags;
  uint8_t* diff;
  uint32_t ref_id, chkpt_id;
};

// flags -> ascending ids of changed chunks, written straight into the diff
struct FlagVal {
  const uint8_t* f;
  __device__ __forceinline__ uint64_t operator()(uint64_t c) const { return f[c] ? 1ull : 0ull; }
};
struct IdEmit {
  uint8_t* diff;
  __device__ __forceinline__ void operator()(uint64_t c, uint64_t ex, uint64_t v) const {
    if (v) *reinterpret_cast<uint32_t*>(diff + 32 + 4 * ex) = (uint32_t)c;
  }
};

// header_t (include/utils.hpp:29-37) of the .basic checkpoint
__global__ void noalloc_header_kernel(NoAllocArgs a, const uint64_t* total) {
  uint32_t* h = reinterpret_cast<uint32_t*>(a.diff);
  const uint32_t F = (uint32_t)*total;
  h[0] = a.ref_id;
  h[1] = a.chkpt_id;
  h[2] = (uint32_t)a.len;
  h[3] = (uint32_t)(a.len >> 32);
  h[4] = a.cs;
  h[5] = F;
  h[6] = 0;
  h[7] = 0;
}

// data section: slot k holds changed chunk ids[k]; the short last chunk is
// padded with zeros (src/basic_approach.cpp:84-114)
__global__ void noalloc_copy_kernel(NoAllocArgs a, const uint64_t* total) {
  const uint64_t F = *total;
  const uint32_t* ids = reinterpret_cast<const uint32_t*>(a.diff + 32);
  uint8_t* dst = a.diff + 32 + 4 * F;
  const uint64_t nbytes = F * a.cs;
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nbytes; b += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t k = b / a.cs, within = b - k * a.cs;
    const uint64_t src = (uint64_t)ids[k] * a.cs + within;
    dst[b] = src < a.len ? a.data[src] : 0;
  }
}

uint8_t* scratch_on_current_device(int* err) {
  // the device address of the scratch array, looked up once per device
  static uint8_t* addr[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { *err = 1; return nullptr; }
  if (!addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) { *err = 1; return nullptr; }
    addr[dev] = static_cast<uint8_t*>(p);
  }
  *err = 0;
  return addr[dev];
}

int fail(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

}  // namespace
}  // namespace mtc

extern "C" int mtc_basic_checkpoint_noalloc(int hash, const void* dev_data, uint64_t len, uint32_t chunk_size,
                                            void* dev_digests, uint32_t ref_id, uint32_t chkpt_id, int first,
                                            void* dev_diff, uint64_t diff_capacity, uint64_t* diff_len,
                                            void* cuda_stream) {
  using namespace mtc;
  if (!dev_data || !dev_digests || !dev_diff || !diff_len || len == 0 || chunk_size == 0)
    return fail(MTC_EINVAL, "bad argument");
  if (hash != MTC_HASH_MURMUR3 && hash != MTC_HASH_MD5) return fail(MTC_EINVAL, "unknown hash");
  const uint64_t n = (len + chunk_size - 1) / chunk_size;
  if (n > kNoAllocMaxChunks) return fail(MTC_ENOTSUP, "more than 4194304 chunks: beyond the fixed scratch of this entry point");
  const uint64_t worst = 32 + n * (4 + (uint64_t)chunk_size);
  if (diff_capacity < worst) return fail(MTC_EINVAL, "diff buffer smaller than 32 + chunks * (4 + chunk_size) bytes");
  if ((reinterpret_cast<uintptr_t>(dev_diff) & 3) != 0) return fail(MTC_EINVAL, "diff buffer not 4-byte aligned");
  int e = 0;
  uint8_t* scratch = scratch_on_current_device(&e);
  if (e) return fail(MTC_ECUDA, "cannot resolve the scratch array on this device");
  uint8_t* flags = scratch;
  uint64_t* tiles = reinterpret_cast<uint64_t*>(scratch + kNoAllocMaxChunks);
  uint64_t* total = tiles + kNoAllocTiles;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);

  // 1. digests, comparison with the previous ones, changed flags
  LeafArgs la;
  la.data = static_cast<const uint8_t*>(dev_data);
  la.len = len;
  la.cs = chunk_size;
  la.n_chunks = (uint32_t)n;
  la.prev = static_cast<Digest*>(dev_digests);
  la.labels = flags;
  la.hash_kind = hash;
  la.epi = EPI_BASIC;
  la.basic_first = first ? 1 : 0;
  TmaCache cache;  // host-side descriptor only
  cudaError_t ce = launch_leaves(la, &cache, s);
  // 2. ascending ids of the changed chunks, straight into the diff
  NoAllocArgs a{la.data, len, chunk_size, (uint32_t)n, flags, static_cast<uint8_t*>(dev_diff), ref_id, chkpt_id};
  if (ce == cudaSuccess) ce = grid_scan(FlagVal{flags}, IdEmit{a.diff}, nullptr, n, tiles, total, s);
  // 3. header and chunk data
  if (ce == cudaSuccess) {
    noalloc_header_kernel<<<1, 1, 0, s>>>(a, total);
    noalloc_copy_kernel<<<num_sms() * 8, 256, 0, s>>>(a, total);
    note_launch(2);
    ce = cudaGetLastError();
  }
  uint64_t F = 0;
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&F, total, sizeof(F), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return fail(MTC_ECUDA, cudaGetErrorString(ce));
  *diff_len = 32 + F * (4 + (uint64_t)chunk_size);
  return MTC_OK;
}
