// mtc_internal.hpp -- host-side declarations shared by the translation units
// of the library (kernel launchers and their argument blocks).  Not part of
// the public interface (see include/mtcheck.h and include/mtcheck/*.hpp).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda.h>

#include "mtc_common.cuh"

namespace mtc {

// Per-chunk epilogue of the leaf kernel.
enum LeafEpi : int {
  EPI_HASH = 0,   // write the digest only
  EPI_TREE = 1,   // TreeDeduplicator leaves (src/tree_approach.cpp:57-94, :309-351)
  EPI_LIST = 2,   // ListDeduplicator::dedup_data (src/list_approach.cpp:38-61)
  EPI_BASIC = 3,  // BasicDeduplicator::dedup_data (src/basic_approach.cpp:25-46)
};

// Per-checkpoint values that kernels read from device memory, so that one
// launch sequence (or a captured graph) serves every checkpoint of a chain.
// Epochs used in one checkpoint: epoch (leaf inserts), epoch + 1 (first-
// occurrence forest), epoch + 2 (the baseline's insert-every-node pass).
struct StepParams {
  uint32_t cur;          // current_id
  uint32_t baseline_id;  // reference checkpoint written into the header
  uint32_t epoch;
  uint32_t pad;
};
constexpr uint32_t kEpochsPerCheckpoint = 3;

struct LeafArgs {
  const uint8_t* data = nullptr;  // device buffer being checkpointed
  uint64_t len = 0;               // bytes
  uint32_t cs = 0;                // chunk size
  uint32_t n_chunks = 0;          // ceil(len / cs)
  Digest* prev = nullptr;         // per-chunk digest of the previous checkpoint (tree leaves or hash list)
  uint8_t* labels = nullptr;      // per-chunk label / changed flag out
  uint32_t* chunk_slot = nullptr; // map slot of each changed-list entry (by list position)
  Digest* out = nullptr;          // EPI_HASH output
  DigestMap map{};
  const StepParams* sp = nullptr; // current checkpoint id and launch epoch (device)
  uint32_t leaf_base = 0;         // node id of chunk 0 (N-1 for the tree, 0 for the list)
  uint32_t* err = nullptr;        // device error word
  uint32_t* changed_list = nullptr;  // chunks whose digest changed (tree, list)
  uint32_t* changed_count = nullptr;
  uint32_t* demoted = nullptr;    // set to 1 when a first occurrence is demoted (tree; may be null)
  uint32_t* dup_list = nullptr;   // changed-list positions that met a duplicate inserted by the same launch
  uint32_t* dup_count = nullptr;  // appends (at most the changed chunks)
  uint32_t dup_cap = 0;
  int hash_kind = HASH_MURMUR3;
  int epi = EPI_HASH;
  int basic_first = 0;            // basic approach with current_id == 0: every chunk changed
  // Fault injection for the failure-detection tests: the TMA producer issues
  // no copy, so every consumer's bounded wait runs out after `spin_limit`
  // polls and the launch ends with DERR_SPIN, no copy in flight.  0 in
  // every normal launch.
  uint32_t stall = 0;
  uint32_t spin_limit = 0;        // 0: kMbarSpinLimit
};


// Cached TMA descriptor for one (buffer, length, chunk size).
struct TmaCache {
  const void* ptr = nullptr;
  uint64_t len = 0;
  uint32_t cs = 0;
  int width = 0;
  int rows = 0;
  CUtensorMap map;
};

// Launch shape of the leaf hashing kernel.  Every choice gives the same
// digests and labels; only the speed differs.
//   rows        -- chunks per CTA tile (TMA box height): 128 or 256
//   ctas_per_sm -- resident CTAs per SM of the persistent grid (0: the most
//                  that fit in shared memory, at most 3)
//   direct      -- 1: every thread loads its own chunk from global memory
//                  instead of the TMA-staged shared-memory pipeline
//   threads_per_chunk -- 1: one thread hashes one chunk (the pipelines
//                  above); 32: one warp per chunk, its lanes loading the
//                  chunk together into shared memory and one lane hashing it
//                  (chunks of 1 to 4096 bytes)
struct LeafTune {
  int rows = 256;
  int ctas_per_sm = 0;
  int direct = 0;
  int threads_per_chunk = 1;
};
// Default shape per digest, measured at 4 GiB / 512 B: Murmur3 tiles of 128
// rows, two CTAs per SM (0.652 ms against 0.691 for 256 rows); MD5, whose
// hashing is ALU-bound, 256 rows and as many CTAs as fit (0.948 ms).
inline LeafTune default_leaf_tune(int hash_kind) {
  return hash_kind == HASH_MD5 ? LeafTune{256, 0, 0} : LeafTune{128, 2, 0};
}

// Launch the leaf hashing kernel(s) over every chunk.  Uses the TMA pipeline
// for chunk sizes that are a multiple of 128 bytes (or 16/32/64) on 16-byte
// aligned buffers, and a thread-per-chunk kernel otherwise and for the tail.
cudaError_t launch_leaves(const LeafArgs& a, TmaCache* cache, cudaStream_t s, const LeafTune& tune = LeafTune{});
// The leaf pass of many deduplicators in one persistent launch (a batch):
// one record per member (its TMA descriptor with boxes of kBatchRows rows,
// its leaf arguments) and a work queue of (member, tile) items.
constexpr int kBatchRows = 128;
struct MemberLeaf {  // aligned as CUtensorMap
  CUtensorMap map;
  LeafArgs la;
  uint32_t n_full, W, xsteps, pad;
};
static_assert(alignof(MemberLeaf) % 64 == 0, "a TMA descriptor in global memory is 64-byte aligned");
struct BatchLeafParams {
  const MemberLeaf* members;
  const uint2* items;   // (member, tile), largest first
  uint32_t nitems;
  uint32_t spin_limit;  // 0: the default bound
  uint32_t* head;       // next item to claim, zero before every launch
};
// Fills a member's record from its leaf arguments; false when the member's
// leaves cannot go through the batched launch (chunk size other than 64 or a
// multiple of 128 bytes, an input not 16-byte aligned, no full chunk).
bool batch_leaf_member(MemberLeaf* out, const LeafArgs& a);
// Kernel node parameters of the batched leaf launch (args: one slot).
cudaError_t batch_leaf_node_params(const BatchLeafParams& p, cudaKernelNodeParams* kp, void** args);
// The leaf kernel for chunks [c0, c1) only, one thread per chunk.
cudaError_t launch_leaf_range(const LeafArgs& a, uint32_t c0, uint32_t c1, cudaStream_t s);

// Tree / list: map inserts of the changed chunks collected by launch_leaves,
// then the lowest-offset demotion (src/tree_approach.cpp:356-369; for the
// list a changed chunk is a first occurrence only if it owns its digest).
cudaError_t launch_leaf_inserts(const LeafArgs& a, cudaStream_t s);

int num_sms();

// Small device results to pinned host memory, written by a kernel through the
// memory's device mapping instead of copied: copies of a few bytes would
// queue on the copy engines behind large transfers of other streams (an
// upload, another process's spill).  Up to three (src, dst, words) segments;
// dst is the device alias of pinned memory (host_alias).
struct Readback {
  const uint32_t* src[3];
  uint32_t* dst[3];
  uint32_t words[3];
};
cudaError_t launch_readback(const Readback& r, cudaStream_t s);
// The device address of pinned host memory (the same pointer under unified
// addressing).
void* host_alias(void* pinned);

// Kernel launch with programmatic stream serialization (see pdl_enter): the
// kernel may be scheduled while its predecessor finishes, hiding the launch
// gap between the dependent kernels of a checkpoint.  Off when MTCHECK_PDL=0,
// and while a thread holds a PdlSuppress (captures that become child graphs).
bool pdl_enabled();
struct PdlSuppress {
  PdlSuppress();
  ~PdlSuppress();
};
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                            Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
// Running count of kernel launches issued by the library (all handles).
void note_launch(uint32_t n = 1);
uint64_t launch_count();

// Kernels that read the checkpointed buffer itself, by argument layout: a
// captured launch sequence follows a new input pointer by updating exactly
// these nodes.  Registered once per kernel by its launch site.
enum : int {
  INPUT_NONE = 0,
  INPUT_LEAF_TMA = 1,     // (const CUtensorMap, LeafArgs, uint32_t)
  INPUT_LEAF_DIRECT = 2,  // (LeafArgs, uint32_t, uint32_t)
  INPUT_GATHER = 3,       // (GatherArgs)
  INPUT_PARAMS = 4,       // (StepParams, StepParams*, uint32_t*): the step values
};
void register_input_kernel(const void* func, int kind);
int input_kernel_kind(const void* func);
// The descriptor launch_leaves gives the TMA leaf kernel for this buffer and
// launch shape (in c->map); false when TMA does not apply.
bool input_tmap(TmaCache* c, const uint8_t* data, uint64_t len, uint32_t cs, const LeafTune& tune);
// Message returned by mtc_last_error() on this thread.
void set_last_error(const char* msg);

}  // namespace mtc
