// noalloc.cu -- a checkpoint entry point that allocates no memory.
//
// Who needs it: code that runs where allocating is not allowed or not safe.
// An out-of-memory handler that wants to save the application's state has, by
// definition, no memory left to ask for; a signal or crash handler that takes
// a last checkpoint on the way down must not enter an allocator that may hold
// a lock or be corrupt; and a runtime whose memory pool already owns the whole
// GPU, or a custom allocator checkpointing its own arena, cannot call
// cudaMalloc without recursing into itself.  Such callers still own the
// buffers they hand over.
//
// What it does: the basic approach (src/basic_approach.cpp:14-143) without a
// deduplicator object.  The caller owns the per-chunk digests of the previous
// checkpoint (updated in place) and a device output buffer that receives the
// .basic incremental checkpoint: header, ids of the changed chunks in
// ascending order, and their data.  The bytes are the same as those of a
// basic-approach deduplicator that has seen the same sequence of buffers.
//
// Scratch: one changed-flag byte per chunk, one scan word per 4096 chunks, the
// count of changed chunks and a device error word, all in the file-scope
// device array below.  Every GPU that loads the library keeps this array
// (kNoAllocScratchBytes, about 4 MiB) until the process exits.  All calls
// share it: each call rewrites everything it reads and clears its error word
// first, and calls that run at the same time on the GPU (different streams or
// threads) race on it, so the caller must serialise them.
#include <atomic>
#include <cstring>
#include <mutex>

#include "../../include/mtcheck.h"
#include "mtc_internal.hpp"
#include "mtc_scan.cuh"

namespace mtc {
namespace {

constexpr uint64_t kNoAllocMaxChunks = 1ull << 22;                    // 4 Mi chunks
constexpr uint64_t kNoAllocTiles = (kNoAllocMaxChunks / kScanTile + 2) & ~1ull;  // scan words (even count)
// [flags: kNoAllocMaxChunks bytes][tile sums: kNoAllocTiles u64]
// [changed count: u64][error word: u32][pad: u32]
constexpr uint64_t kNoAllocTailOffset = kNoAllocMaxChunks + 8 * kNoAllocTiles;
constexpr uint64_t kNoAllocScratchBytes = kNoAllocTailOffset + 16;
static_assert(kNoAllocTailOffset % 16 == 0, "count and error word share one aligned 16-byte read");

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocArgs {
  const uint8_t* data;
  uint64_t len;
  uint32_t cs, n;
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

// Data section: slot k holds changed chunk ids[k]; the short last chunk is
// padded with zeros (src/basic_approach.cpp:84-114).  One warp per slot; whole
// chunks of a multiple of 16 bytes from a 16-byte aligned buffer move as
// 16-byte loads (the slots are only 4-byte aligned in general: the data
// section starts after 4 bytes per id).
__global__ void noalloc_copy_kernel(NoAllocArgs a, const uint64_t* total) {
  const uint64_t F = *total;
  const uint32_t* ids = reinterpret_cast<const uint32_t*>(a.diff + 32);
  uint8_t* dst0 = a.diff + 32 + 4 * F;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const bool vec = (a.cs % 16 == 0) && ((reinterpret_cast<uintptr_t>(a.data) & 15) == 0);
  const bool dst16 = (reinterpret_cast<uintptr_t>(dst0) & 15) == 0;
  for (uint64_t k = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < F; k += nwarps) {
    const uint64_t off = (uint64_t)ids[k] * a.cs;
    const uint64_t avail = off < a.len ? (a.len - off < a.cs ? a.len - off : a.cs) : 0;
    uint8_t* dst = dst0 + k * a.cs;
    if (vec && avail == a.cs) {
      const uint4* src = reinterpret_cast<const uint4*>(a.data + off);
      for (uint32_t u = lane; u < a.cs / 16; u += 32) {
        const uint4 v = __ldg(src + u);
        if (dst16) {
          *reinterpret_cast<uint4*>(dst + 16 * u) = v;
        } else {
          uint32_t* d = reinterpret_cast<uint32_t*>(dst + 16 * u);
          d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
        }
      }
    } else {
      for (uint32_t b = lane; b < a.cs; b += 32) dst[b] = b < avail ? a.data[off + b] : 0;
    }
  }
}

// Set-up, once per device: the device address of the scratch array.  In host
// code `g_noalloc_scratch` names a host-side stand-in, not device memory, so
// kernels are given the address that cudaGetSymbolAddress returns for the
// current device.  The address stays valid until the process exits or the
// device is reset (cudaDeviceReset unloads the module; the cached value is
// then stale).
constexpr int kMaxDevices = 64;
std::atomic<uint8_t*> g_scratch_addr[kMaxDevices];
std::mutex g_setup_mu;

int scratch_on_current_device(uint8_t** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MTC_ECUDA;
  uint8_t* p = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    p = g_scratch_addr[dev].load(std::memory_order_relaxed);
    if (!p) {
      void* q = nullptr;
      if (cudaGetSymbolAddress(&q, g_noalloc_scratch) != cudaSuccess || !q) return MTC_ECUDA;
      p = static_cast<uint8_t*>(q);
      g_scratch_addr[dev].store(p, std::memory_order_release);
    }
  }
  *out = p;
  return MTC_OK;
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
  if (n > kNoAllocMaxChunks)
    return fail(MTC_ENOTSUP, "more than 4194304 chunks: beyond the fixed scratch of this entry point");
  const uint64_t worst = 32 + n * (4 + (uint64_t)chunk_size);
  if (diff_capacity < worst) return fail(MTC_EINVAL, "diff buffer smaller than 32 + chunks * (4 + chunk_size) bytes");
  if ((reinterpret_cast<uintptr_t>(dev_diff) & 3) != 0) return fail(MTC_EINVAL, "diff buffer not 4-byte aligned");
  if ((reinterpret_cast<uintptr_t>(dev_digests) & 15) != 0)
    return fail(MTC_EINVAL, "digest buffer not 16-byte aligned");
  uint8_t* scratch = nullptr;
  if (scratch_on_current_device(&scratch) != MTC_OK)
    return fail(MTC_ECUDA, "cannot resolve the scratch array on this device");
  uint8_t* flags = scratch;
  uint64_t* tiles = reinterpret_cast<uint64_t*>(scratch + kNoAllocMaxChunks);
  uint64_t* total = reinterpret_cast<uint64_t*>(scratch + kNoAllocTailOffset);
  uint32_t* err = reinterpret_cast<uint32_t*>(total + 1);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);

  // the error word starts at zero; everything else is rewritten before use
  cudaError_t ce = cudaMemsetAsync(err, 0, sizeof(uint32_t), s);
  // 1. digests, comparison with the previous ones, changed flags
  LeafArgs la;
  la.data = static_cast<const uint8_t*>(dev_data);
  la.len = len;
  la.cs = chunk_size;
  la.n_chunks = (uint32_t)n;
  la.prev = static_cast<Digest*>(dev_digests);
  la.labels = flags;
  la.err = err;
  la.hash_kind = hash;
  la.epi = EPI_BASIC;
  la.basic_first = first ? 1 : 0;
  TmaCache cache;  // host-side descriptor only
  if (ce == cudaSuccess) ce = launch_leaves(la, &cache, s);
  // 2. ascending ids of the changed chunks, straight into the diff
  NoAllocArgs a{la.data, len, chunk_size, (uint32_t)n, static_cast<uint8_t*>(dev_diff), ref_id, chkpt_id};
  if (ce == cudaSuccess) ce = grid_scan(FlagVal{flags}, IdEmit{a.diff}, nullptr, n, tiles, total, s);
  // 3. header and chunk data
  if (ce == cudaSuccess) {
    noalloc_header_kernel<<<1, 1, 0, s>>>(a, total);
    noalloc_copy_kernel<<<num_sms() * 8, 256, 0, s>>>(a, total);
    note_launch(2);
    ce = cudaGetLastError();
  }
  // changed count and error word in one read
  uint64_t tail[2] = {0, 0};
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(tail, total, sizeof(tail), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return fail(MTC_ECUDA, cudaGetErrorString(ce));
  const uint32_t derr = (uint32_t)tail[1];
  if (derr & DERR_SPIN) return fail(MTC_ETIMEOUT, "bounded device wait expired");
  if (derr) return fail(MTC_EINTERNAL, "device error");
  *diff_len = 32 + tail[0] * (4 + (uint64_t)chunk_size);
  return MTC_OK;
}
