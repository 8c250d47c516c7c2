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
  uint32_t root_fo, max_key, ok, reserved;
};

struct ForestArgs {
  Digest* tree;
  uint8_t* labels;
  uint8_t* rflag;
  DigestMap map;
  uint32_t cur, epoch;
  uint32_t* err;
  int hash_kind;
};

struct GatherArgs {
  int approach;
  const uint8_t* data;
  uint64_t len;
  uint32_t cs, N, M, cur, baseline_id;
  const Digest* digests;  // tree heap (by node) or hash list (by chunk)
  DigestMap map;
  uint32_t* err;
  const uint32_t* fo_list;
  const uint32_t* sh_list;
  uint64_t* fo_val;
  uint32_t *reg_chunk, *reg_slot, *reg_len;
  uint32_t *sh_key, *sh_prev;
  uint32_t *hist, *rep;
  uint64_t* sort_mat;
  uint64_t *scan_scratch, *scan_total, *scan_scratch2, *scan_total2;
  uint8_t* stage;
  uint64_t stage_cap;
  Layout* lay;
};

cudaError_t launch_fo_level(const ForestArgs& a, uint32_t beg, uint32_t end, cudaStream_t s);
cudaError_t launch_dup_level(const ForestArgs& a, uint32_t beg, uint32_t end, int baseline, cudaStream_t s);
cudaError_t launch_insert_level(const ForestArgs& a, uint32_t beg, uint32_t end, cudaStream_t s);
cudaError_t launch_root_compaction(const uint8_t* labels, const uint8_t* rflag, uint32_t N, uint32_t M, int ascending,
                                   uint32_t* fo_list, uint32_t* sh_list, Layout* lay, uint64_t* scan_scratch,
                                   uint64_t* scan_total, cudaStream_t s);
cudaError_t launch_chunk_compaction(const uint8_t* labels, uint32_t n_chunks, int basic, uint32_t* fo_list,
                                    uint32_t* sh_list, Layout* lay, uint64_t* scan_scratch, uint64_t* scan_total,
                                    cudaStream_t s);
// Assemble the diff into g.stage; max_entries bounds F and S (N + 1).
cudaError_t launch_assemble(const GatherArgs& g, uint64_t max_entries, cudaStream_t s);
// Rebuild `from` into the empty table `to` (capacity change), preserving values.
cudaError_t launch_map_rehash(const DigestMap& from, uint64_t from_cap, const DigestMap& to, uint32_t* err,
                              cudaStream_t s);

}  // namespace mtc
