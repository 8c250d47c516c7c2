// engine.hpp -- the device-side state of one deduplicator and the host code
// that drives its kernels.  One Engine serves every approach of the
// reference (full / basic / list / tree, and the tree with the serial
// reference labelling); the public C++ classes and the C ABI wrap it.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>

#include "mtc_common.cuh"
#include "mtc_gather.hpp"
#include "mtc_internal.hpp"

namespace mtc {

// Return a status from an Engine member when a CUDA call fails.
#define MTC_CUDA_R(call)                                                                                   \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess)                                                                                 \
      return fail(e_ == cudaErrorMemoryAllocation ? ST_ENOMEM : ST_ECUDA,                                  \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                                      \
  } while (0)

struct RestartScratch;
void destroy_restart_scratch(RestartScratch* r);

// DedupMode values of the reference (include/utils.hpp:39-49).
enum : int { MODE_FULL = 1, MODE_BASIC = 2, MODE_LIST = 3, MODE_TREE = 4, MODE_TREE_LOW_OFFSET_REF = 5, MODE_TREE_LOW_OFFSET = 6 };

// Public status codes (mirrored in include/mtcheck.h).
enum : int { ST_OK = 0, ST_EINVAL = 1, ST_ECORRUPT = 2, ST_ENOMEM = 3, ST_ETIMEOUT = 4, ST_ECUDA = 5, ST_EINTERNAL = 6, ST_ENOTSUP = 7 };

struct HeaderHost {  // header_t, include/utils.hpp:29-37
  uint32_t ref_id, chkpt_id;
  uint64_t datalen;
  uint32_t chunk_size, num_first_ocur, num_prior_chkpts, num_shift_dupl;
};
static_assert(sizeof(HeaderHost) == 32, "header_t is 32 bytes");

// Device bytes of an engine's state for a buffer of `len` bytes in chunks of
// `cs`: digests, labels, lists, digest map at load <= 3/4, staging for the
// largest diff (the server's admission and a batch's reservation use it).
inline uint64_t estimate_state_bytes(int mode, uint64_t len, uint32_t cs) {
  const uint64_t N = (len + cs - 1) / cs, M = 2 * N;
  if (mode == MODE_FULL) return len + 64;
  const bool tree = mode == MODE_TREE || mode == MODE_TREE_LOW_OFFSET || mode == MODE_TREE_LOW_OFFSET_REF;
  const uint64_t nd = tree ? M : N;
  uint64_t slots = 1;
  while (slots < nd * 4 / 3 + 1) slots <<= 1;
  const uint64_t map = mode == MODE_BASIC ? 0 : slots * 2 * sizeof(MapSlot);
  return nd * (sizeof(Digest) + 2) + N * 64 + map + (N + 1) * (cs + 12) + (1u << 20);
}

// MTCHECK_SERVER_TRACE=1: every host step timed by a StepTimer that takes
// longer than 20 ms is reported on stderr with its name and duration (the
// served worker's steps and the parts of a restart's enqueue).
inline bool trace_on() {
  static const bool v = [] {
    const char* e = std::getenv("MTCHECK_SERVER_TRACE");
    return e && e[0] == '1';
  }();
  return v;
}
struct StepTimer {
  const char* what;
  uint32_t id;
  std::chrono::steady_clock::time_point t0;
  StepTimer(const char* w, uint32_t i) : what(w), id(i) {
    if (trace_on()) t0 = std::chrono::steady_clock::now();
  }
  ~StepTimer() {
    if (!trace_on()) return;
    const double dt = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (dt > 20.0) std::fprintf(stderr, "mtc-trace: %s (%u) took %.1f ms\n", what, id, dt);
  }
};

// Grow-only device array.  With a memory pool set, allocation and release
// are stream-ordered (cudaMallocFromPoolAsync / cudaFreeAsync on the stream
// of the call) and never wait for the device; without one, cudaMalloc and
// cudaFree.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;  // elements
  cudaMemPool_t pool = nullptr;
  cudaStream_t owner = nullptr;  // stream of the last pool allocation
  cudaError_t ensure(size_t want, cudaStream_t s, bool keep = false) {
    if (want <= n && p) return cudaSuccess;
    T* q = nullptr;
    const size_t bytes = sizeof(T) * (want ? want : 1);
    cudaError_t e = pool ? cudaMallocFromPoolAsync(reinterpret_cast<void**>(&q), bytes, pool, s)
                         : cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return e;
    if (keep && p && n) cudaMemcpyAsync(q, p, sizeof(T) * n, cudaMemcpyDeviceToDevice, s);
    if (p) {
      if (pool) {
        cudaFreeAsync(p, s);
      } else {
        cudaStreamSynchronize(s);
        cudaFree(p);
      }
    }
    p = q;
    n = want;
    owner = s;
    return cudaSuccess;
  }
  void release(cudaStream_t s = nullptr) {
    if (p) {
      if (pool) cudaFreeAsync(p, s ? s : owner);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
  }
  ~DevBuf() { release(); }
};

class Engine {
 public:
  Engine(int mode, int hash_kind, uint32_t chunk_size);
  ~Engine();

  // checkpoint(header_t&, ...) of the reference: the diff is assembled in
  // device memory; current_id is not advanced.
  int checkpoint(const uint8_t* dev_data, uint64_t len, bool make_baseline, HeaderHost* header);
  // The same checkpoint in three parts, for callers that batch engines or
  // capture the work into a CUDA graph:
  //   prepare      -- validation and every allocation; may synchronise
  //   stage_params -- host-side step values (id, epochs) for the next enqueue
  //   enqueue      -- stream-ordered work only (capturable once prepared):
  //                   reads the step values, writes the diff and the layout
  //                   readback into pinned host memory
  //   complete     -- after the stream has drained: error mapping, counters
  // id_headroom sizes the per-source-checkpoint tables for that many further
  // checkpoints, so that one captured sequence serves them all.
  int prepare(const uint8_t* dev_data, uint64_t len, bool make_baseline, uint32_t id_headroom);
  void stage_params();
  int enqueue(const uint8_t* dev_data, uint64_t len, bool timed);
  int complete(uint64_t len, HeaderHost* header);
  // Fingerprint of everything a captured sequence depends on.
  uint64_t signature(const uint8_t* dev_data, uint64_t len) const;
  // The same without the input's address (only its alignment).
  uint64_t shape_signature(const uint8_t* dev_data, uint64_t len) const;
  bool fresh() const { return fresh_; }
  // True once after prepare() put work on the engine's stream that leaves
  // every device pointer in place (so the signature does not show it).
  // The single-call path replays its launch sequence as a CUDA graph,
  // captured at the first incremental checkpoint and again whenever the
  // signature changes (on by default; a Batch never uses it).
  void set_own_graph(bool on);
  bool own_graph() const { return own_graph_; }
  // Replay an incremental checkpoint as one graph without the phase events
  // between its segments; its timers and phase times then read 0.
  void set_untimed(bool on);
  bool untimed() const { return untimed_; }
  // Batch members read their step values from the pinned block at run time.
  void set_params_from_host(bool on) { params_by_value_ = !on; }
  bool take_stream_work() {
    const bool w = stream_work_;
    stream_work_ = false;
    return w;
  }
  void set_max_load(double f) { max_load_ = f; }
  double max_load() const { return max_load_; }
  void set_leaf_tune(const LeafTune& t) { leaf_tune_ = t; }
  const LeafTune& leaf_tune() const { return leaf_tune_; }
  uint64_t map_capacity() const { return map_cap_; }
  // Free device buffers replaced by map growth; call once the stream has
  // drained (the single-call path does it itself).
  void release_retired();
  uint64_t device_bytes() const;
  // Frees the restart buffers (stream-ordered); the next restart allocates
  // and clears them again.
  void release_restart_scratch();
  uint64_t restart_scratch_bytes() const;
  // The 32-byte headers of a chain resident in device memory, read on the
  // handle's stream by one gather kernel and one copy (zeros for a diff
  // shorter than a header).
  int read_headers(const std::vector<const uint8_t*>& ptrs, const std::vector<uint64_t>& lens,
                   std::vector<HeaderHost>& out);
  // Stream-ordered allocation from `pool` for every device buffer of this
  // engine (set before the first checkpoint).
  void set_pool(cudaMemPool_t pool);
  // Move the persistent state (chunk digests, digest map) to pinned host
  // memory and free every device buffer; restore it before the next call.
  // The copies run on the engine's stream; spill_to_host() returns once they
  // are issued, the host copy is valid after the stream drains.
  bool spilled() const { return spilled_; }
  uint64_t spill_bytes() const;
  int spill_to_host(uint8_t* host);
  int restore_from_host(const uint8_t* host);

  // Copy the staged diff to host memory (pinned or pageable).
  int copy_diff(void* host, uint64_t cap);
  const uint8_t* diff_device() const;
  uint64_t diff_len() const { return diff_len_; }
  // restart(View, chain, logname, id): `dev_diffs` are device-resident copies
  // of the chain (the main one is index `id`).
  int restart(uint8_t* dev_out, uint64_t len, const std::vector<const uint8_t*>& dev_diffs,
              const std::vector<uint64_t>& lens, const std::vector<HeaderHost>& headers, uint32_t id);
  // The same in two parts: stream-ordered work, then (after the stream has
  // drained) timers and error mapping.  The chain must stay valid until then.
  int restart_enqueue(uint8_t* dev_out, uint64_t len, const std::vector<const uint8_t*>& dev_diffs,
                      const std::vector<uint64_t>& lens, const std::vector<HeaderHost>& headers, uint32_t id);
  int restart_complete();

  int mode() const { return mode_; }
  int hash_kind() const { return hash_kind_; }
  uint32_t chunk_size() const { return cs_; }
  uint32_t current_id = 0;
  uint32_t baseline_id = 0;
  uint64_t data_len = 0;
  uint32_t num_first_ocur = 0, num_shift_dupl = 0, num_prior_chkpts = 0;
  uint64_t datasizes[2] = {0, 0};
  double timers[4] = {0, 0, 0, 0};          // setup, compare, gather, copy-to-host (seconds)
  double restart_timers[2] = {0, 0};        // copy, total
  double phase_times[3] = {0, 0, 0};        // leaf hashing kernel, forest + roots, diff assembly (s)
  uint32_t last_device_error = 0;
  std::string last_error;

  cudaStream_t stream() const { return stream_; }
  void set_stream(cudaStream_t s) { stream_ = s; }
  // For engines on a non-blocking stream of the library (batch members,
  // server processes): single calls first wait for the work already issued
  // to the legacy default stream, where callers usually write their buffers.
  void set_order_after_legacy(bool on) { order_after_legacy_ = on; }
  int order_inputs();
  uint32_t launches() const { return launches_; }
  // A batch takes over the leaf pass of its members' captured sequences:
  // while a hook is set, the sequence calls it where it would launch the
  // leaf kernels.
  struct LeafHook {
    virtual int on_leaves(Engine* e, const LeafArgs& la, cudaStream_t s) = 0;
    virtual ~LeafHook() {}
  };
  void set_leaf_hook(LeafHook* h) { leaf_hook_ = h; }
  // The engine's own leaf launch (its descriptor cache and launch shape).
  cudaError_t launch_own_leaves(const LeafArgs& la, cudaStream_t s) { return launch_leaves(la, &tma_, s, leaf_tune_); }
  // Fault injection for tests: the next n checkpoints run eagerly with the
  // chunk-hashing kernel's copy producer silent, so its bounded waits run
  // out and the checkpoint fails with ST_ETIMEOUT.
  void inject_stall(uint32_t n) { stall_left_ = n; }
  // After a device timeout the digest state may be partly updated: the next
  // checkpoint is taken as a baseline.
  bool needs_baseline() const { return need_baseline_; }

 private:
  int fail(int code, const std::string& msg);
  int ensure_state(uint32_t N, bool fresh, uint32_t id_headroom);
  int ensure_map(uint64_t want_entries, bool reset);
  int ensure_sort(uint32_t K);
  int run_tree(const uint8_t* data, uint64_t len, bool baseline_path);
  int run_list_basic(const uint8_t* data, uint64_t len);
  GatherArgs gather_args(const uint8_t* data, uint64_t len);

  int mode_, hash_kind_;
  uint32_t cs_;
  cudaStream_t stream_ = nullptr;
  bool allocated_ = false;
  bool fresh_ = false, baseline_path_ = false, timed_ = true, order_after_legacy_ = false, spilled_ = false;
  cudaMemPool_t pool_ = nullptr;
  template <class F> void for_each_buf(F f);
  double max_load_ = 0.75;
  LeafTune leaf_tune_{};
  uint32_t N_ = 0, M_ = 0;
  bool own_graph_ = true;
  bool untimed_ = false;
  // the captured sequence, cut at the timing marks: the event recorded
  // before each segment (or -1) and the segment's graph (null when empty)
  struct OwnSeg {
    int mark;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
  };
  std::vector<OwnSeg> own_segs_;
  // kernel nodes that read the input buffer, with their captured arguments
  struct InputNode {
    size_t seg;
    cudaGraphNode_t node;
    int kind;
    cudaKernelNodeParams p;
    CUtensorMap tmap;
    LeafArgs la;
    uint32_t u[2];
    GatherArgs ga;
    StepParams* sp_dev;  // INPUT_PARAMS: the kernel's pointer arguments
    uint32_t* err_dev;
  };
  std::vector<InputNode> input_nodes_;
  const uint8_t* own_data_ = nullptr;  // input pointer the graphs currently read
  cudaStream_t cap_stream_ = nullptr;  // private stream the sequence is captured on
  uint64_t own_sig_ = 0, own_kernels_ = 0;
  int retarget_own(const uint8_t* data, uint64_t len);
  int update_own_params();
  bool seg_capture_ = false;  // enqueue runs under a capture cut at each mark
  int seg_mark_ = -1;
  std::vector<std::pair<int, cudaGraph_t>> seg_graphs_;
  int replay_own(const uint8_t* data, uint64_t len);
  int mark(int i);
  void drop_own_graph();
  bool stream_work_ = false;
  LeafHook* leaf_hook_ = nullptr;
  uint32_t stall_left_ = 0;
  bool stall_now_ = false, need_baseline_ = false;
  uint32_t epoch_ = 0;
  uint64_t map_cap_ = 0;
  uint32_t map_size_host_ = 0;
  uint32_t launches_ = 0;

  DevBuf<Digest> digests_;     // tree heap (M) or hash list (N)
  DevBuf<uint8_t> labels_, rflag_;
  DevBuf<uint32_t> chunk_slot_, changed_list_, changed_count_;
  DevBuf<MapSlot> slots_;
  DevBuf<uint32_t> map_size_, err_;
  DevBuf<uint32_t> fo_list_, sh_list_, reg_chunk_, reg_slot_, reg_len_, sh_key_, sh_prev_, hist_, rep_, rank_;
  DevBuf<uint64_t> fo_val_, sort_mat_, scan_, scan_total_, scan2_, scan_total2_;
  DevBuf<uint8_t> stage_;
  DevBuf<Layout> lay_;
  DevBuf<StepParams> sp_;
  StepParams* sp_host_ = nullptr;   // pinned
  Layout* lay_host_ = nullptr;      // pinned
  uint32_t* err_host_ = nullptr;    // pinned [err, map size]
  bool params_by_value_ = true;     // false for batch members (their graphs copy sp_host_)
  uint64_t diff_len_ = 0, diff_pad_ = 0;
  TmaCache tma_;
  cudaEvent_t ev_[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  RestartScratch* rs_ = nullptr;  // restart buffers, created on first use
  // restart: a second stream for the work that does not depend on the main
  // sequence (clears, the chain tables beside the main scatter, the copy of
  // resolved chunk ranges), and the events that fork and join it
  cudaStream_t rside_ = nullptr;
  cudaEvent_t rev_[12] = {};
  // pinned staging of a restart's chain descriptors (kept when the restart
  // tables are released: freeing pinned memory waits for the device), and
  // the event after their last upload
  void* rdi_host_ = nullptr;
  size_t rdi_host_bytes_ = 0;
  cudaEvent_t rdi_ev_ = nullptr;
  DevBuf<uint8_t> hdr_dev_;         // read_headers: gathered headers
 public:
  // A host chain copied to device memory for a restart (the staging path of
  // mtc_restart); kept between restarts, released with the restart tables.
  DevBuf<uint8_t> restart_stage;
 private:
  uint8_t* hdr_host_ = nullptr;     // pinned copy of them
  size_t hdr_host_cap_ = 0;
  std::vector<void*> retired_;    // replaced map tables awaiting cudaFree
  uint64_t spill_nd_ = 0, spill_cap_ = 0;
  bool restart_raw_ = false;
};

}  // namespace mtc
