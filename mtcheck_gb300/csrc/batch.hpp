// batch.hpp -- many deduplicators checkpointed together.
//
// A Batch owns one Engine per buffer (any approach, hash and chunk size), each
// on its own CUDA stream.  One call checkpoints every member:
//   * a step in which some member starts a new baseline runs eagerly, every
//     member's work issued on its own stream so that they overlap;
//   * every other step replays one CUDA graph holding every member's launch
//     sequence as an independent child graph, in one launch on the origin
//     stream.  A member's sequence reads the per-step values (checkpoint id,
//     epochs) from pinned host memory, so it is captured once and replayed
//     until that member's device buffers move (map growth, a new input
//     pointer); only that member is captured again and its child node of
//     the instantiated parent updated (the parent is rebuilt when the
//     update is refused).
// A step starts after all work already issued to the legacy default stream
// (where the inputs are usually written); inputs written on other streams
// must be synchronised by the caller.
// Every member's diff, header and counters are exactly those of the same
// engine driven one call at a time: the launch sequence is the same, only the
// issue mechanism differs.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "engine.hpp"

namespace mtc {

struct BatchStats {
  uint64_t steps = 0;
  uint64_t captures = 0;
  uint64_t graph_nodes = 0;       // nodes of all members' graphs
  uint64_t batched_leaf_items = 0;  // work items of the batched leaf launch (0: none)
  uint32_t batched_leaf_members = 0;
  uint64_t kernels_per_step = 0;  // kernel launches issued (eager) or held in the graphs
  double last_device_ms = 0;      // fork to join of the last step, CUDA events on the origin stream
  double last_call_ms = 0;        // host wall time of the last checkpoint() call
  double host_ms[5] = {0, 0, 0, 0, 0};  // prepare, capture, issue, wait, complete
  int last_used_graph = 0;
};

class Batch : public Engine::LeafHook {
 public:
  Batch();
  ~Batch();
  // Add a member; returns its index or -1.
  int add(int mode, int hash_kind, uint32_t chunk_size);
  uint32_t size() const { return (uint32_t)engs_.size(); }
  Engine* member(uint32_t i) { return i < engs_.size() ? engs_[i] : nullptr; }
  // One checkpoint of every member (the reference's checkpoint(data, len,
  // diff_h, make_baseline) overload per member, current_id advanced).
  int checkpoint(const uint8_t* const* data, const uint64_t* lens, bool make_baseline, uint64_t* diff_lens);
  // Grow the members' memory pool, now, to hold their state for buffers of
  // these lengths (allocated once and returned to the pool, which keeps it),
  // so that the first checkpoint allocates without growing the pool.
  int reserve(const uint64_t* lens, uint64_t* bytes);
  void set_use_graph(bool g) { use_graph_ = g; }
  void set_id_headroom(uint32_t h) { headroom_ = h ? h : 1; }
  // off: every member launches its own leaf kernels in its graph (no
  // batched leaf launch)
  void set_leaf_batching(bool on) { leaf_batching_ = on; }
  const BatchStats& stats() const { return stats_; }
  std::string last_error;
  // Engine::LeafHook: a member's captured sequence reaches its leaf pass
  int on_leaves(Engine* e, const LeafArgs& la, cudaStream_t s) override;

 private:
  int fail(int code, const std::string& msg);
  int capture_member(size_t i, const uint8_t* data, uint64_t len);
  int build_parent();
  void drop_parent();
  void drop_graph();

  std::vector<Engine*> engs_;
  std::vector<cudaStream_t> streams_;
  std::vector<cudaEvent_t> joins_;
  cudaStream_t origin_ = nullptr;
  cudaMemPool_t pool_ = nullptr;  // stream-ordered allocations of every member
  cudaEvent_t fork_ = nullptr, in_ = nullptr, t0_ = nullptr, t1_ = nullptr;
  // each member's captured sequence, cut at its leaf pass when the batched
  // leaf launch takes it over: pre_ (up to the leaves) and post_ (after);
  // otherwise the whole sequence in pre_
  std::vector<cudaGraph_t> pre_, post_;
  std::vector<char> in_kernel_;      // the member's leaves run in the batched launch
  std::vector<MemberLeaf> recs_;     // their records (host copy)
  std::vector<uint64_t> sigs_, nodes_, kernels_;
  size_t cur_ = 0;                   // member being captured
  // step graph: [head reset, members' pre_] -> batched leaf launch -> members' post_
  cudaGraph_t parent_ = nullptr;
  cudaGraphExec_t parent_exec_ = nullptr;
  MemberLeaf* members_dev_ = nullptr;
  uint2* items_dev_ = nullptr;
  uint32_t* head_dev_ = nullptr;
  size_t members_cap_ = 0, items_cap_ = 0;
  BatchLeafParams leaf_params_{};
  bool use_graph_ = true, leaf_batching_ = false;
  uint32_t headroom_ = 64;
  BatchStats stats_;
};

// Autotuner: times the leaf-kernel launch shapes and map load factors on a
// synthetic buffer of the given length (seeded fill, a few percent of chunks
// rewritten per step) and returns the fastest.  Results are cached per
// (approach, hash, chunk size, power-of-two length bucket) for the process.
struct TuneResult {
  LeafTune leaf;
  double max_load = 0.75;
  double ms = 0;        // best incremental-checkpoint device time
  double default_ms = 0;
  int candidates = 0;
};
int autotune(int mode, int hash_kind, uint32_t chunk_size, uint64_t len, bool use_cache, TuneResult* out,
             std::string* err);

}  // namespace mtc
