// mtc_gather.hpp -- argument blocks and launchers of the forest, compaction
// and diff-assembly kernels (gather_kernels.cu) and of the map maintenance
// kernels.  Internal to the library.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mtc_common.cuh"
#include "mtc_internal.hpp"

namespace mtc {

enum : int { APPROACH_TREE = 0, APPROACH_LIST = 1, APPROACH_BASIC = 2 };
constexpr uint32_t kSortTile = 4096;

// Device-resident description of one assembled diff.  Offsets are relative to
// the first header byte, which sits at stage + pad (pad makes the data section
// 16-byte aligned in device memory).
struct Layout {
  uint32_t F, S, P, num_distinct;  // FO entries, shift entries, source checkpoints, valid FO regions
  uint64_t chunk_counter;          // chunk slots in the data section
  uint64_t pad, data_off, table_off, pairs_off, diff_len;
  uint64_t size_data, size_meta;   // the reference's datasizes pair
  uint32_t root_fo, max_key, ok, nkeys;  // nkeys: distinct sort keys of the shift entries
  uint32_t sort_n, sort_tiles;            // nkeys * sort tiles; tiles of kSortTile shift entries
};

struct ForestArgs {
  Digest* tree;
  uint8_t* labels;
  uint8_t* rflag;  // root flags at canonical positions (M-1 bytes)
  DigestMap map;
  const StepParams* sp;  // cur, epochs (device)
  uint32_t* err;
  int hash_kind;
  int ascending;   // canonical order: 0 = deeper levels first (serial push order), 1 = ascending node id
  uint32_t D;      // depth of node M-1
  uint64_t sizeD;  // nodes on depth D
  // Incremental checkpoints: word that is 0 when no leaf was demoted to a
  // shifted duplicate of a digest first seen in this checkpoint.  Then no
  // shifted pair can hash to a digest inserted by the first-occurrence pass
  // (its leaves would share a digest with a first occurrence, whose digest is
  // new), so both passes run in one traversal.  Null: two passes.
  const uint32_t* fuse_gate;
  uint32_t* ins_queue;  // first-occurrence nodes awaiting their map insert (N entries)
  uint32_t* ins_count;
};

// Position of node x (>= 1) in the canonical root order.
__host__ __device__ __forceinline__ uint64_t canon_pos(const ForestArgs& a, uint32_t x) {
  if (a.ascending) return (uint64_t)x - 1;
#ifdef __CUDA_ARCH__
  const uint32_t d = 31 - __clz(x + 1);
#else
  uint32_t d = 0;
  while (((2ull << d) - 1) <= (uint64_t)x) d++;
#endif
  const uint64_t fp = d == a.D ? 0 : a.sizeD + ((1ull << a.D) - (2ull << d));
  return fp + (x - ((1ull << d) - 1));
}

struct GatherArgs {
  int approach;
  const uint8_t* data;
  uint64_t len;
  uint32_t cs, N, M;
  const StepParams* sp;   // cur, baseline_id (device)
  uint32_t k_cap;         // capacity of hist / rep / rank (checkpoint ids + 1)
  const Digest* digests;  // tree heap (by node) or hash list (by chunk)
  DigestMap map;
  uint32_t* err;
  const uint32_t* fo_list;
  const uint32_t* sh_list;
  uint64_t* fo_val;
  uint32_t *reg_chunk, *reg_slot, *reg_len;
  uint32_t *sh_key, *sh_prev;
  uint32_t *hist, *rep, *rank;
  uint64_t* sort_mat;
  uint64_t *scan_scratch, *scan_total, *scan_scratch2, *scan_total2;
  uint8_t* stage;
  uint64_t stage_cap;
  Layout* lay;
};

// All levels of one forest pass in a few launches (9 levels each).
// pass 0 = first-occurrence forest, 1 = duplicate forest.
cudaError_t launch_forest(const ForestArgs& a, int pass, int baseline, uint32_t N, cudaStream_t s);
cudaError_t launch_root_compaction(const ForestArgs& fa, uint32_t N, uint32_t M, uint32_t* fo_list,
                                   uint32_t* sh_list, Layout* lay, uint64_t* scan_scratch, uint64_t* scan_total,
                                   cudaStream_t s);
cudaError_t launch_chunk_compaction(const uint8_t* labels, uint32_t n_chunks, int basic, uint32_t* fo_list,
                                    uint32_t* sh_list, Layout* lay, uint64_t* scan_scratch, uint64_t* scan_total,
                                    cudaStream_t s);
// Assemble the diff into g.stage; max_entries bounds F and S (N + 1).
cudaError_t launch_assemble(const GatherArgs& g, uint64_t max_entries, cudaStream_t s);
// Rebuild `from` into the empty table `to` (capacity change), preserving values.
cudaError_t launch_map_rehash(const DigestMap& from, uint64_t from_cap, const DigestMap& to, uint32_t* err,
                              cudaStream_t s);
// Every entry's epoch set to 0 (before the epoch counter restarts).
cudaError_t launch_map_rebase(const DigestMap& m, uint64_t cap, cudaStream_t s);

}  // namespace mtc
