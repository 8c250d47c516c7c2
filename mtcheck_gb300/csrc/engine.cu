// engine.cu -- host orchestration of one deduplicator: device state, map
// growth, the per-checkpoint launch sequence and the readback of the diff
// layout.  Mirrors TreeDeduplicator / ListDeduplicator / BasicDeduplicator /
// FullDeduplicator::checkpoint(header_t&, ...) (src/tree_approach.cpp:1578-1689,
// src/list_approach.cpp:843-931, src/basic_approach.cpp:468-549,
// src/full_approach.cpp:14-77).
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "engine.hpp"
#include "mtc_scan.cuh"

namespace mtc {

static __global__ void set_word_kernel(uint32_t* p, uint32_t v) { *p = v; }

// The step values as a kernel argument, and the error word cleared: nothing
// crosses the host link, so a large transfer already queued there (the next
// input's upload, say) cannot delay the checkpoint -- a host-to-device copy
// would wait behind it on the copy engine, and a kernel reading mapped host
// memory behind it on the link.  A replayed graph gets each step's values
// by an update of this node (Engine::replay_own).
static __global__ void params_in_kernel(StepParams p, StepParams* dev, uint32_t* err) {
  pdl_enter();
  if (threadIdx.x == 0) {
    *dev = p;
    *err = 0;
  }
}

// Polls of an injected stall's bounded waits (about a millisecond).
constexpr uint32_t kInjectedSpinLimit = 1u << 14;

static __global__ void readback_kernel(Readback r) {
  pdl_enter();
#pragma unroll
  for (int k = 0; k < 3; k++)
    for (uint32_t i = threadIdx.x; i < r.words[k]; i += blockDim.x) r.dst[k][i] = r.src[k][i];
}

cudaError_t launch_readback(const Readback& r, cudaStream_t s) {
  launch_k(readback_kernel, 1, 32, 0, s, r);
  note_launch();
  return cudaGetLastError();
}

void* host_alias(void* pinned) {
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, pinned, 0) != cudaSuccess) {
    cudaGetLastError();
    return pinned;
  }
  return d;
}

static uint64_t next_pow2(uint64_t v) {
  uint64_t c = 1;
  while (c < v) c <<= 1;
  return c;
}

Engine::Engine(int mode, int hash_kind, uint32_t chunk_size)
    : mode_(mode), hash_kind_(hash_kind), cs_(chunk_size), leaf_tune_(default_leaf_tune(hash_kind)) {
  for (auto& e : ev_) cudaEventCreate(&e);
  cudaMallocHost(&lay_host_, sizeof(Layout));
  cudaMallocHost(&err_host_, 2 * sizeof(uint32_t));
  cudaMallocHost(&sp_host_, sizeof(StepParams));
  std::memset(lay_host_, 0, sizeof(Layout));
  std::memset(sp_host_, 0, sizeof(StepParams));
  // test hook: start the launch epochs near their limit to exercise the rebase
  if (const char* e = std::getenv("MTCHECK_EPOCH_START")) epoch_ = (uint32_t)std::strtoul(e, nullptr, 10);
}

Engine::~Engine() {
  if (stream_) cudaStreamSynchronize(stream_); else cudaDeviceSynchronize();
  drop_own_graph();
  if (cap_stream_) cudaStreamDestroy(cap_stream_);
  if (rside_) {
    cudaStreamSynchronize(rside_);
    cudaStreamDestroy(rside_);
  }
  for (auto& e : ev_) if (e) cudaEventDestroy(e);
  for (auto& e : rev_) if (e) cudaEventDestroy(e);
  if (lay_host_) cudaFreeHost(lay_host_);
  if (err_host_) cudaFreeHost(err_host_);
  if (sp_host_) cudaFreeHost(sp_host_);
  if (hdr_host_) cudaFreeHost(hdr_host_);
  if (rdi_ev_) cudaEventDestroy(rdi_ev_);
  if (rdi_host_) cudaFreeHost(rdi_host_);
  release_retired();
  destroy_restart_scratch(rs_);
}

int Engine::fail(int code, const std::string& msg) {
  last_error = msg;
  return code;
}

#define MTC_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return fail(e_ == cudaErrorMemoryAllocation ? ST_ENOMEM : ST_ECUDA, \
                                       std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
#define MTC_TRY(call)         \
  do {                        \
    const int rc_ = (call);   \
    if (rc_) return rc_;      \
  } while (0)

int Engine::ensure_map(uint64_t want_entries, bool reset) {
  // load factor <= max_load after the worst-case number of inserts of one
  // checkpoint (3/4 unless tuned)
  uint64_t need = next_pow2(std::max<uint64_t>(1024, (uint64_t)((double)want_entries / max_load_) + 1));
  if (reset) {
    if (slots_.n < need || slots_.n > 4 * need) {
      slots_.release();
      MTC_CUDA(slots_.ensure(need, stream_));
    }
    map_cap_ = slots_.n;
    MTC_CUDA(cudaMemsetAsync(slots_.p, kMapFill, sizeof(MapSlot) * map_cap_, stream_));
    MTC_CUDA(cudaMemsetAsync(map_size_.p, 0, sizeof(uint32_t), stream_));
    map_size_host_ = 0;
    return ST_OK;
  }
  if (map_cap_ >= need) return ST_OK;
  DevBuf<MapSlot> fresh;
  MTC_CUDA(fresh.ensure(need, stream_));
  MTC_CUDA(cudaMemsetAsync(fresh.p, kMapFill, sizeof(MapSlot) * need, stream_));
  MTC_CUDA(cudaMemsetAsync(map_size_.p, 0, sizeof(uint32_t), stream_));
  DigestMap from{slots_.p, map_cap_ - 1, map_size_.p};
  DigestMap to{fresh.p, need - 1, map_size_.p};
  MTC_CUDA(launch_map_rehash(from, map_cap_, to, err_.p, stream_));
  // the old table is freed after the rehash: stream-ordered from a pool,
  // otherwise once the stream has drained (release_retired), because
  // cudaFree here would wait for the whole device
  if (pool_) cudaFreeAsync(slots_.p, stream_);
  else retired_.push_back(slots_.p);
  slots_.p = fresh.p;
  slots_.n = fresh.n;
  fresh.p = nullptr;
  fresh.n = 0;
  map_cap_ = need;
  return ST_OK;
}

void Engine::release_retired() {
  for (void* p : retired_) cudaFree(p);
  retired_.clear();
}

int Engine::ensure_sort(uint32_t K) {
  // capacities grow in powers of two so that a growing checkpoint id does not
  // reallocate on every call
  K = (uint32_t)next_pow2(std::max<uint32_t>(K, 64));
  const uint64_t T = (uint64_t)(N_ + 1 + kSortTile - 1) / kSortTile + 1;
  MTC_CUDA(hist_.ensure(K, stream_));
  MTC_CUDA(rep_.ensure(K, stream_));
  MTC_CUDA(rank_.ensure(K, stream_));
  MTC_CUDA(sort_mat_.ensure((size_t)K * T, stream_));
  MTC_CUDA(scan2_.ensure((size_t)K * T / kScanTile + 2, stream_));
  // staging buffer: pad + header + metadata + data
  const uint64_t stage = 64 + 32 + 12ull * (N_ + 1) + 8ull * K + (uint64_t)(N_ + 1) * cs_;
  MTC_CUDA(stage_.ensure(stage, stream_));
  return ST_OK;
}

int Engine::ensure_state(uint32_t N, bool fresh, uint32_t id_headroom) {
  const uint32_t M = 2 * N - 1;
  const bool tree = mode_ == MODE_TREE || mode_ == MODE_TREE_LOW_OFFSET || mode_ == MODE_TREE_LOW_OFFSET_REF;
  if (fresh) {
    N_ = N;
    M_ = M;
    const size_t nd = tree ? M : N;
    MTC_CUDA(digests_.ensure(nd, stream_));
    MTC_CUDA(cudaMemsetAsync(digests_.p, 0, sizeof(Digest) * nd, stream_));
    MTC_CUDA(labels_.ensure(nd, stream_));
    MTC_CUDA(rflag_.ensure(tree ? M : 1, stream_));
    MTC_CUDA(chunk_slot_.ensure(N, stream_));
    MTC_CUDA(changed_list_.ensure(N, stream_));
    MTC_CUDA(changed_count_.ensure(4, stream_));  // [changed chunks, leaves demoted, forest inserts, duplicate notes]
    MTC_CUDA(map_size_.ensure(1, stream_));
    MTC_CUDA(err_.ensure(1, stream_));
    MTC_CUDA(fo_list_.ensure(N + 1, stream_));
    MTC_CUDA(sh_list_.ensure(N + 1, stream_));
    MTC_CUDA(fo_val_.ensure(N + 1, stream_));
    MTC_CUDA(reg_chunk_.ensure(N + 1, stream_));
    MTC_CUDA(reg_slot_.ensure(N + 1, stream_));
    MTC_CUDA(reg_len_.ensure(N + 1, stream_));
    MTC_CUDA(sh_key_.ensure(N + 1, stream_));
    MTC_CUDA(sh_prev_.ensure(N + 1, stream_));
    // tile sums: scans of 4096 entries over max(M, N+1), or of 512 regions over N+1
    MTC_CUDA(scan_.ensure(std::max<size_t>((size_t)(std::max(M, N + 1) + kScanTile - 1) / kScanTile,
                                           ((size_t)N + 1 + 511) / 512) + 2, stream_));
    MTC_CUDA(scan_total_.ensure(1, stream_));
    MTC_CUDA(scan_total2_.ensure(1, stream_));
    MTC_CUDA(lay_.ensure(1, stream_));
    MTC_CUDA(sp_.ensure(1, stream_));
    if (mode_ != MODE_BASIC) {
      // room for the baseline's inserts and the worst case of the next
      // checkpoint, so that the first incremental checkpoint does not grow it
      int rc = ensure_map(2ull * (tree ? M : N), true);
      if (rc) return rc;
    }
    allocated_ = true;
  }
  if (mode_ != MODE_BASIC) {
    int rc = ensure_map((uint64_t)map_size_host_ + (tree ? M_ : N_), false);
    if (rc) return rc;
    // map entries keep their epoch in 26 bits: before the counter gets
    // there, every entry goes back to epoch 0 (older than any launch to come)
    if (epoch_ + kEpochsPerCheckpoint >= kEpochLimit) {
      if (map_cap_) MTC_CUDA(launch_map_rebase(DigestMap{slots_.p, map_cap_ - 1, map_size_.p}, map_cap_, stream_));
      epoch_ = 0;
      stream_work_ = true;
    }
  }
  return ensure_sort(current_id + 1 + id_headroom);
}

GatherArgs Engine::gather_args(const uint8_t* data, uint64_t len) {
  GatherArgs g{};
  g.approach = mode_ == MODE_LIST ? APPROACH_LIST : mode_ == MODE_BASIC ? APPROACH_BASIC : APPROACH_TREE;
  g.data = data;
  g.len = len;
  g.cs = cs_;
  g.N = N_;
  g.M = M_;
  g.sp = sp_.p;
  g.k_cap = (uint32_t)hist_.n;
  g.digests = digests_.p;
  g.map = DigestMap{slots_.p, map_cap_ ? map_cap_ - 1 : 0, map_size_.p};
  g.err = err_.p;
  g.fo_list = fo_list_.p;
  g.sh_list = sh_list_.p;
  g.fo_val = fo_val_.p;
  g.reg_chunk = reg_chunk_.p;
  g.reg_slot = reg_slot_.p;
  g.reg_len = reg_len_.p;
  g.sh_key = sh_key_.p;
  g.sh_prev = sh_prev_.p;
  g.hist = hist_.p;
  g.rep = rep_.p;
  g.rank = rank_.p;
  g.sort_mat = sort_mat_.p;
  g.scan_scratch = scan_.p;
  g.scan_total = scan_total_.p;
  g.scan_scratch2 = scan2_.p;
  g.scan_total2 = scan_total2_.p;
  g.stage = stage_.p;
  g.stage_cap = stage_.n;
  g.lay = lay_.p;
  return g;
}

int Engine::run_tree(const uint8_t* data, uint64_t len, bool baseline_path) {
  const uint32_t N = N_, M = M_;
  DigestMap map{slots_.p, map_cap_ - 1, map_size_.p};
  LeafArgs la;
  la.data = data;
  la.len = len;
  la.cs = cs_;
  la.n_chunks = N;
  la.prev = digests_.p + (N - 1);
  la.labels = labels_.p + (N - 1);
  la.chunk_slot = chunk_slot_.p;
  la.map = map;
  la.sp = sp_.p;
  la.leaf_base = N - 1;
  la.err = err_.p;
  la.hash_kind = hash_kind_;
  la.epi = EPI_TREE;
  la.changed_list = changed_list_.p;
  la.changed_count = changed_count_.p;
  la.demoted = changed_count_.p + 1;
  // the first-occurrence root list is free until the root compaction
  la.dup_list = fo_list_.p;
  la.dup_count = changed_count_.p + 3;
  la.dup_cap = (uint32_t)fo_list_.n;
  if (stall_now_) {
    la.stall = 1;
    la.spin_limit = kInjectedSpinLimit;
  }
  MTC_CUDA(cudaMemsetAsync(changed_count_.p, 0, 4 * sizeof(uint32_t), stream_));
  if (leaf_hook_) MTC_TRY(leaf_hook_->on_leaves(this, la, stream_));
  else MTC_CUDA(launch_leaves(la, &tma_, stream_, leaf_tune_));
  if (timed_) MTC_TRY(mark(4));
  MTC_CUDA(launch_leaf_inserts(la, stream_));

  ForestArgs fa{};
  fa.tree = digests_.p;
  fa.labels = labels_.p;
  fa.rflag = rflag_.p;
  fa.map = map;
  fa.sp = sp_.p;
  fa.err = err_.p;
  fa.hash_kind = hash_kind_;
  fa.ascending = mode_ == MODE_TREE_LOW_OFFSET_REF ? 1 : 0;
  fa.D = 0;
  while (((2ull << fa.D) - 1) <= (uint64_t)(M - 1)) fa.D++;  // depth of node M-1
  fa.sizeD = (uint64_t)M - ((1ull << fa.D) - 1);
  // an incremental checkpoint without demoted leaves runs both passes in one
  // traversal (the launches of the duplicate pass then return at once)
  fa.fuse_gate = baseline_path ? nullptr : la.demoted;
  // the changed-chunk list is free once the leaf inserts are done: it queues
  // the forest's first-occurrence inserts
  fa.ins_queue = changed_list_.p;
  fa.ins_count = changed_count_.p + 2;
  MTC_CUDA(launch_forest(fa, 0, 0, N, stream_));                         // first-occurrence forest
  MTC_CUDA(launch_forest(fa, 1, baseline_path ? 1 : 0, N, stream_));  // duplicate forest
  MTC_CUDA(launch_root_compaction(fa, N, M, fo_list_.p, sh_list_.p, lay_.p, scan_.p, scan_total_.p, stream_));
  return ST_OK;
}

int Engine::run_list_basic(const uint8_t* data, uint64_t len) {
  LeafArgs la;
  la.data = data;
  la.len = len;
  la.cs = cs_;
  la.n_chunks = N_;
  la.prev = digests_.p;
  la.labels = labels_.p;
  la.chunk_slot = chunk_slot_.p;
  la.map = DigestMap{slots_.p, map_cap_ ? map_cap_ - 1 : 0, map_size_.p};
  la.sp = sp_.p;
  la.leaf_base = 0;
  la.err = err_.p;
  la.hash_kind = hash_kind_;
  la.epi = mode_ == MODE_LIST ? EPI_LIST : EPI_BASIC;
  la.basic_first = current_id == 0 ? 1 : 0;  // never true in a captured sequence
  la.changed_list = changed_list_.p;
  la.changed_count = changed_count_.p;
  la.dup_list = fo_list_.p;  // free until the chunk compaction
  la.dup_count = changed_count_.p + 3;
  la.dup_cap = (uint32_t)fo_list_.n;
  if (stall_now_) {
    la.stall = 1;
    la.spin_limit = kInjectedSpinLimit;
  }
  MTC_CUDA(cudaMemsetAsync(changed_count_.p, 0, 4 * sizeof(uint32_t), stream_));
  if (leaf_hook_) MTC_TRY(leaf_hook_->on_leaves(this, la, stream_));
  else MTC_CUDA(launch_leaves(la, &tma_, stream_, leaf_tune_));
  if (timed_) MTC_TRY(mark(4));
  if (mode_ == MODE_LIST) MTC_CUDA(launch_leaf_inserts(la, stream_));
  MTC_CUDA(launch_chunk_compaction(labels_.p, N_, mode_ == MODE_BASIC ? 1 : 0, fo_list_.p, sh_list_.p, lay_.p, scan_.p,
                                   scan_total_.p, stream_));
  return ST_OK;
}

int Engine::prepare(const uint8_t* data, uint64_t len, bool make_baseline, uint32_t id_headroom) {
  if (!data || len == 0) return fail(ST_EINVAL, "empty buffer");
  if (spilled_) return fail(ST_EINVAL, "state spilled to host: restore it first");
  if (need_baseline_) make_baseline = true;  // the last checkpoint timed out on the device
  const uint64_t n64 = (len + cs_ - 1) / cs_;
  if (n64 >= (1ull << 31)) return fail(ST_ENOTSUP, "more than 2^31 chunks");
  const uint32_t N = (uint32_t)n64;
  fresh_ = make_baseline || !allocated_;
  if (mode_ != MODE_FULL && !fresh_ && len != data_len)
    return fail(ST_EINVAL, "buffer length changed without a new baseline");
  if (mode_ == MODE_FULL) {
    MTC_CUDA(stage_.ensure(len + 64, stream_));
    allocated_ = true;
  } else {
    int rc = ensure_state(N, fresh_, id_headroom);
    if (rc) return rc;
  }
  data_len = len;
  // TreeLowOffsetRef follows include/reference_impl.hpp:16-132, which has no
  // baseline special case; the tree modes follow dedup_data_baseline for
  // checkpoint 0 and every requested baseline (src/tree_approach.cpp:1644-1653)
  baseline_path_ = mode_ != MODE_TREE_LOW_OFFSET_REF && (current_id == 0 || make_baseline);
  if (current_id == 0 || make_baseline) baseline_id = current_id;
  return ST_OK;
}

void Engine::stage_params() {
  // the previous checkpoint of this engine has completed, so the pinned
  // block is free to rewrite
  sp_host_->cur = current_id;
  sp_host_->baseline_id = baseline_id;
  sp_host_->epoch = epoch_ + 1;
  epoch_ += kEpochsPerCheckpoint;
}

int Engine::enqueue(const uint8_t* data, uint64_t len, bool timed) {
  timed_ = timed;
  if (timed) MTC_TRY(mark(0));
  if (mode_ == MODE_FULL) {
    // FullDeduplicator: the checkpoint is the raw buffer (src/full_approach.cpp:66-72)
    if (timed) MTC_TRY(mark(1));
    if (timed) MTC_TRY(mark(2));
    MTC_CUDA(cudaMemcpyAsync(stage_.p, data, len, cudaMemcpyDeviceToDevice, stream_));
    if (timed) MTC_TRY(mark(3));
    return ST_OK;
  }
  if (params_by_value_) {
    static const bool reg = (register_input_kernel(reinterpret_cast<const void*>(params_in_kernel), INPUT_PARAMS), true);
    (void)reg;
    launch_k(params_in_kernel, 1, 32, 0, stream_, *sp_host_, sp_.p, err_.p);
    note_launch();
    MTC_CUDA(cudaGetLastError());
  } else {
    // a batch member: its sequence, replayed inside the batch's graph, copies
    // the step values staged in the pinned block
    MTC_CUDA(cudaMemcpyAsync(sp_.p, sp_host_, sizeof(StepParams), cudaMemcpyHostToDevice, stream_));
    MTC_CUDA(cudaMemsetAsync(err_.p, 0, sizeof(uint32_t), stream_));
  }
  if (timed) MTC_TRY(mark(1));
  int rc = (mode_ == MODE_LIST || mode_ == MODE_BASIC) ? run_list_basic(data, len) : run_tree(data, len, baseline_path_);
  if (rc) return rc;
  if (timed) MTC_TRY(mark(2));
  MTC_CUDA(launch_assemble(gather_args(data, len), (uint64_t)N_ + 1, stream_));
  if (timed) MTC_TRY(mark(3));
  // results (layout, error word, map size) written to pinned memory by a
  // kernel, not queued on a copy engine behind other streams' transfers
  static_assert(sizeof(Layout) % 4 == 0, "layout copied as words");
  Readback rb{};
  rb.src[0] = reinterpret_cast<const uint32_t*>(lay_.p);
  rb.dst[0] = static_cast<uint32_t*>(host_alias(lay_host_));
  rb.words[0] = sizeof(Layout) / 4;
  rb.src[1] = err_.p;
  rb.dst[1] = static_cast<uint32_t*>(host_alias(err_host_));
  rb.words[1] = 1;
  if (map_size_.p) {
    rb.src[2] = map_size_.p;
    rb.dst[2] = rb.dst[1] + 1;
    rb.words[2] = 1;
  }
  MTC_CUDA(launch_readback(rb, stream_));
  return ST_OK;
}

int Engine::order_inputs() {
  if (!order_after_legacy_) return ST_OK;
  MTC_CUDA(cudaEventRecord(ev_[5], cudaStreamLegacy));
  MTC_CUDA(cudaStreamWaitEvent(stream_, ev_[5], 0));
  return ST_OK;
}

void Engine::drop_own_graph() {
  for (auto& sg : own_segs_) {
    if (sg.exec) cudaGraphExecDestroy(sg.exec);
    if (sg.graph) cudaGraphDestroy(sg.graph);
  }
  own_segs_.clear();
  input_nodes_.clear();
  own_sig_ = 0;
  own_data_ = nullptr;
}

// Points the captured sequence at another input buffer of the same length
// and alignment: the leaf kernels' descriptor and pointer, the chunk gather's
// pointer (no other kernel reads the input).
int Engine::retarget_own(const uint8_t* data, uint64_t len) {
  for (auto& in : input_nodes_) {
    void* args[3] = {nullptr, nullptr, nullptr};
    if (in.kind == INPUT_PARAMS) continue;
    if (in.kind == INPUT_LEAF_TMA) {
      if (!input_tmap(&tma_, data, len, cs_, leaf_tune_)) return fail(ST_ECUDA, "tensor map for the new input");
      in.tmap = tma_.map;
      in.la.data = data;
      args[0] = &in.tmap;
      args[1] = &in.la;
      args[2] = &in.u[0];
    } else if (in.kind == INPUT_LEAF_DIRECT) {
      in.la.data = data;
      args[0] = &in.la;
      args[1] = &in.u[0];
      args[2] = &in.u[1];
    } else {
      in.ga.data = data;
      args[0] = &in.ga;
    }
    cudaKernelNodeParams q = in.p;
    q.kernelParams = args;
    q.extra = nullptr;
    MTC_CUDA(cudaGraphExecKernelNodeSetParams(own_segs_[in.seg].exec, in.node, &q));
  }
  own_data_ = data;
  return ST_OK;
}

// Gives the captured sequence this step's values (the argument of its first
// kernel).
int Engine::update_own_params() {
  for (auto& in : input_nodes_) {
    if (in.kind != INPUT_PARAMS) continue;
    StepParams sp = *sp_host_;
    void* args[3] = {&sp, &in.sp_dev, &in.err_dev};
    cudaKernelNodeParams q = in.p;
    q.kernelParams = args;
    q.extra = nullptr;
    MTC_CUDA(cudaGraphExecKernelNodeSetParams(own_segs_[in.seg].exec, in.node, &q));
  }
  return ST_OK;
}

void Engine::set_untimed(bool on) {
  if (on != untimed_) drop_own_graph();
  untimed_ = on;
}

void Engine::set_own_graph(bool on) {
  own_graph_ = on;
  if (!on) drop_own_graph();
}

// A timing mark of the launch sequence: an event on the stream, or, while
// the sequence is being captured, the end of one segment and the start of the
// next (an event recorded by a graph cannot be timed, so the events are
// recorded between the segments' launches).
int Engine::mark(int i) {
  if (!seg_capture_) {
    MTC_CUDA(cudaEventRecord(ev_[i], stream_));
    return ST_OK;
  }
  if (untimed_) return ST_OK;  // one graph, no phase events
  cudaGraph_t g = nullptr;
  MTC_CUDA(cudaStreamEndCapture(cap_stream_, &g));
  seg_graphs_.emplace_back(seg_mark_, g);
  seg_mark_ = i;
  MTC_CUDA(cudaStreamBeginCapture(cap_stream_, cudaStreamCaptureModeRelaxed));
  return ST_OK;
}

// The launch sequence of an incremental checkpoint as a few graph launches:
// each replay updates the step values (an argument of the first kernel) and,
// for a new input buffer, the nodes that read the input, so one capture
// serves every checkpoint until a device buffer or the launch shape changes
// (the signature).
int Engine::replay_own(const uint8_t* data, uint64_t len) {
  const uint64_t sig = shape_signature(data, len);
  if (!own_segs_.empty() && sig == own_sig_ && data != own_data_) MTC_TRY(retarget_own(data, len));
  if (own_segs_.empty() || sig != own_sig_) {
    drop_own_graph();
    if (!cap_stream_) MTC_CUDA(cudaStreamCreateWithFlags(&cap_stream_, cudaStreamNonBlocking));
    const uint64_t l0 = launch_count();
    seg_graphs_.clear();
    seg_mark_ = -1;
    MTC_CUDA(cudaStreamBeginCapture(cap_stream_, cudaStreamCaptureModeRelaxed));
    cudaStream_t keep = stream_;
    stream_ = cap_stream_;
    seg_capture_ = true;
    int rc = enqueue(data, len, true);
    seg_capture_ = false;
    stream_ = keep;
    cudaGraph_t g = nullptr;
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(cap_stream_, &st);
    const cudaError_t ee = st == cudaStreamCaptureStatusActive ? cudaStreamEndCapture(cap_stream_, &g) : cudaSuccess;
    if (g) seg_graphs_.emplace_back(seg_mark_, g);
    cudaError_t ie = cudaSuccess;
    if (rc == ST_OK && ee == cudaSuccess) {
      for (auto& sg : seg_graphs_) {
        size_t n = 0;
        cudaGraphGetNodes(sg.second, nullptr, &n);
        cudaGraphExec_t x = nullptr;
        if (n && ie == cudaSuccess) ie = cudaGraphInstantiate(&x, sg.second, 0);
        own_segs_.push_back(OwnSeg{sg.first, sg.second, x});
        sg.second = nullptr;  // owned by own_segs_ (node handles stay valid for updates)
        if (!n || ie != cudaSuccess) continue;
        std::vector<cudaGraphNode_t> nodes(n);
        cudaGraphGetNodes(own_segs_.back().graph, nodes.data(), &n);
        for (cudaGraphNode_t nd : nodes) {
          cudaGraphNodeType ty;
          if (cudaGraphNodeGetType(nd, &ty) != cudaSuccess || ty != cudaGraphNodeTypeKernel) continue;
          InputNode in{};
          if (cudaGraphKernelNodeGetParams(nd, &in.p) != cudaSuccess) continue;
          in.kind = input_kernel_kind(in.p.func);
          if (in.kind == INPUT_NONE) continue;
          in.seg = own_segs_.size() - 1;
          in.node = nd;
          if (in.kind == INPUT_LEAF_TMA) {
            std::memcpy(&in.tmap, in.p.kernelParams[0], sizeof(CUtensorMap));
            std::memcpy(&in.la, in.p.kernelParams[1], sizeof(LeafArgs));
            std::memcpy(&in.u[0], in.p.kernelParams[2], sizeof(uint32_t));
          } else if (in.kind == INPUT_LEAF_DIRECT) {
            std::memcpy(&in.la, in.p.kernelParams[0], sizeof(LeafArgs));
            std::memcpy(&in.u[0], in.p.kernelParams[1], sizeof(uint32_t));
            std::memcpy(&in.u[1], in.p.kernelParams[2], sizeof(uint32_t));
          } else if (in.kind == INPUT_PARAMS) {
            std::memcpy(&in.sp_dev, in.p.kernelParams[1], sizeof(StepParams*));
            std::memcpy(&in.err_dev, in.p.kernelParams[2], sizeof(uint32_t*));
          } else {
            std::memcpy(&in.ga, in.p.kernelParams[0], sizeof(GatherArgs));
          }
          in.p.kernelParams = nullptr;
          input_nodes_.push_back(in);
        }
      }
    }
    for (auto& sg : seg_graphs_)
      if (sg.second) cudaGraphDestroy(sg.second);
    seg_graphs_.clear();
    if (rc != ST_OK || ee != cudaSuccess || ie != cudaSuccess) {
      drop_own_graph();
      cudaGetLastError();
      if (rc != ST_OK) return rc;
      return fail(ST_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ee != cudaSuccess ? ee : ie));
    }
    own_sig_ = sig;
    own_data_ = data;
    own_kernels_ = launch_count() - l0;  // counted while capturing, run by the launches below
  } else {
    MTC_TRY(update_own_params());
    note_launch((uint32_t)own_kernels_);
  }
  for (auto& sg : own_segs_) {
    if (sg.mark >= 0) MTC_CUDA(cudaEventRecord(ev_[sg.mark], stream_));
    if (sg.exec) MTC_CUDA(cudaGraphLaunch(sg.exec, stream_));
  }
  timed_ = !untimed_;
  return ST_OK;
}

int Engine::checkpoint(const uint8_t* data, uint64_t len, bool make_baseline, HeaderHost* header) {
  int rc = prepare(data, len, make_baseline, 0);
  if (rc) return rc;
  if ((rc = order_inputs()) != ST_OK) return rc;
  if (mode_ != MODE_FULL) stage_params();
  stall_now_ = stall_left_ > 0 && mode_ != MODE_FULL;
  if (stall_now_) stall_left_--;
  // a step that allocates (a first checkpoint or a new baseline) runs eagerly,
  // and so does an injected stall (never part of a captured sequence)
  if (own_graph_ && mode_ != MODE_FULL && !fresh_ && !stall_now_) rc = replay_own(data, len);
  else rc = enqueue(data, len, true);
  stall_now_ = false;
  if (rc) return rc;
  MTC_CUDA(cudaStreamSynchronize(stream_));
  release_retired();
  return complete(len, header);
}

// Milliseconds between two of the engine's events; 0 when they cannot be
// timed (the error is consumed, not left for the next call to find).
static float event_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return ms;
}

int Engine::complete(uint64_t len, HeaderHost* header) {
  float ms[3] = {0, 0, 0};
  if (timed_) {
    ms[0] = event_ms(ev_[0], ev_[1]);
    ms[1] = event_ms(ev_[1], ev_[2]);
    ms[2] = event_ms(ev_[2], ev_[3]);
    timers[0] = ms[0] * 1e-3; timers[1] = ms[1] * 1e-3; timers[2] = ms[2] * 1e-3;
  } else {
    timers[0] = timers[1] = timers[2] = 0;
    phase_times[0] = phase_times[1] = phase_times[2] = 0;
  }
  if (mode_ == MODE_FULL) {
    diff_len_ = len;
    diff_pad_ = 0;
    datasizes[0] = len;
    datasizes[1] = 0;
    if (header) std::memset(header, 0, sizeof(*header));
    return ST_OK;
  }
  const Layout& L = *lay_host_;
  last_device_error = err_host_[0];
  if (map_size_.p) map_size_host_ = err_host_[1];
  if (timed_) {
    const float leaf = event_ms(ev_[1], ev_[4]), rest = event_ms(ev_[4], ev_[2]);
    phase_times[0] = leaf * 1e-3; phase_times[1] = rest * 1e-3; phase_times[2] = ms[2] * 1e-3;
  }
  if (last_device_error & DERR_SPIN) {
    // some chunks' digests may already be stored: the next checkpoint starts
    // from scratch as a baseline
    need_baseline_ = true;
    return fail(ST_ETIMEOUT, "bounded device wait expired (the next checkpoint is taken as a baseline)");
  }
  if (last_device_error & (DERR_MAP_FULL | DERR_CAPACITY)) return fail(ST_ENOMEM, "device table or staging buffer full");
  if (last_device_error & DERR_MISSING) return fail(ST_EINTERNAL, "root digest missing from the map");
  if (last_device_error & DERR_SORTKEYS) return fail(ST_ENOTSUP, "more than 1024 distinct source checkpoints in one diff");
  if (!L.ok) return fail(ST_EINTERNAL, "diff layout failed");
  if (fresh_) need_baseline_ = false;
  diff_len_ = L.diff_len;
  diff_pad_ = L.pad;
  num_first_ocur = L.F;
  num_shift_dupl = mode_ == MODE_BASIC ? 0 : L.S;
  num_prior_chkpts = mode_ == MODE_BASIC ? 0 : L.P;
  datasizes[0] = L.size_data;
  datasizes[1] = L.size_meta;
  if (header) {
    header->ref_id = baseline_id;
    header->chkpt_id = current_id;
    header->datalen = len;
    header->chunk_size = cs_;
    header->num_first_ocur = num_first_ocur;
    header->num_prior_chkpts = num_prior_chkpts;
    header->num_shift_dupl = num_shift_dupl;
  }
  return ST_OK;
}

uint64_t Engine::signature(const uint8_t* data, uint64_t len) const {
  // everything a captured launch sequence bakes in: the input, every device
  // buffer, the map and sort capacities, the baseline branch
  return (shape_signature(data, len) ^ (uint64_t)data) * 1099511628211ull;
}

uint64_t Engine::shape_signature(const uint8_t* data, uint64_t len) const {
  // the signature without the input's address, only its alignment (which
  // chooses the kernels that read it): the single-call graph follows a moved
  // input by retarget_own
  const uint64_t v[] = {(uint64_t)data & 15, len, (uint64_t)digests_.p, (uint64_t)labels_.p, (uint64_t)rflag_.p,
                        (uint64_t)chunk_slot_.p, (uint64_t)changed_list_.p, (uint64_t)changed_count_.p,
                        (uint64_t)slots_.p, map_cap_, (uint64_t)map_size_.p, (uint64_t)err_.p, (uint64_t)fo_list_.p,
                        (uint64_t)sh_list_.p, (uint64_t)reg_chunk_.p, (uint64_t)reg_slot_.p, (uint64_t)reg_len_.p,
                        (uint64_t)sh_key_.p, (uint64_t)sh_prev_.p, (uint64_t)hist_.p, hist_.n, (uint64_t)rep_.p,
                        (uint64_t)rank_.p, (uint64_t)fo_val_.p, (uint64_t)sort_mat_.p, sort_mat_.n, (uint64_t)scan_.p,
                        (uint64_t)scan_total_.p, (uint64_t)scan2_.p, (uint64_t)scan_total2_.p, (uint64_t)stage_.p,
                        stage_.n, (uint64_t)lay_.p, (uint64_t)sp_.p, (uint64_t)baseline_path_, (uint64_t)mode_,
                        (uint64_t)leaf_tune_.rows, (uint64_t)leaf_tune_.ctas_per_sm, (uint64_t)leaf_tune_.direct,
                        (uint64_t)leaf_tune_.threads_per_chunk};
  uint64_t h = 1469598103934665603ull;
  for (uint64_t x : v) h = (h ^ x) * 1099511628211ull;
  return h;
}

template <class F>
void Engine::for_each_buf(F f) {
  f(digests_); f(labels_); f(rflag_); f(chunk_slot_); f(changed_list_); f(changed_count_); f(slots_);
  f(map_size_); f(err_); f(fo_list_); f(sh_list_); f(reg_chunk_); f(reg_slot_); f(reg_len_); f(sh_key_);
  f(sh_prev_); f(hist_); f(rep_); f(rank_); f(fo_val_); f(sort_mat_); f(scan_); f(scan_total_); f(scan2_);
  f(scan_total2_); f(stage_); f(lay_); f(sp_);
}

void Engine::set_pool(cudaMemPool_t pool) {
  pool_ = pool;
  for_each_buf([&](auto& b) { b.pool = pool; });
  restart_stage.pool = pool;
}

uint64_t Engine::spill_bytes() const {
  const bool tree = mode_ == MODE_TREE || mode_ == MODE_TREE_LOW_OFFSET || mode_ == MODE_TREE_LOW_OFFSET_REF;
  return sizeof(Digest) * (uint64_t)(tree ? M_ : N_) + sizeof(MapSlot) * map_cap_ + 16;
}

int Engine::spill_to_host(uint8_t* host) {
  if (spilled_) return ST_OK;
  if (!pool_) return fail(ST_ENOTSUP, "spilling needs stream-ordered allocation (a memory pool)");
  if (!allocated_ || mode_ == MODE_FULL) return fail(ST_EINVAL, "nothing to spill");
  const bool tree = mode_ == MODE_TREE || mode_ == MODE_TREE_LOW_OFFSET || mode_ == MODE_TREE_LOW_OFFSET_REF;
  const uint64_t nd = tree ? M_ : N_;  // the digests in use (the buffer may be larger)
  MTC_CUDA(cudaMemcpyAsync(host, digests_.p, sizeof(Digest) * nd, cudaMemcpyDeviceToHost, stream_));
  uint8_t* q = host + sizeof(Digest) * nd;
  if (slots_.p) MTC_CUDA(cudaMemcpyAsync(q, slots_.p, sizeof(MapSlot) * map_cap_, cudaMemcpyDeviceToHost, stream_));
  q += sizeof(MapSlot) * map_cap_;
  std::memcpy(q, &map_size_host_, sizeof(uint32_t));
  spill_nd_ = nd;
  spill_cap_ = map_cap_;
  for_each_buf([&](auto& b) { b.release(stream_); });
  if (rs_) {
    destroy_restart_scratch(rs_);  // stream-ordered frees
    rs_ = nullptr;
  }
  spilled_ = true;
  return ST_OK;
}

int Engine::restore_from_host(const uint8_t* host) {
  if (!spilled_) return ST_OK;
  spilled_ = false;
  const bool tree = mode_ == MODE_TREE || mode_ == MODE_TREE_LOW_OFFSET || mode_ == MODE_TREE_LOW_OFFSET_REF;
  const uint32_t saved_size = [&] { uint32_t v; std::memcpy(&v, host + sizeof(Digest) * spill_nd_ + sizeof(MapSlot) * spill_cap_, 4); return v; }();
  int rc = ensure_state(N_, true, 0);  // every buffer, zeroed; map sized for M
  if (rc) return rc;
  if (mode_ != MODE_BASIC && slots_.n != spill_cap_) {
    slots_.release(stream_);
    MTC_CUDA(slots_.ensure(spill_cap_, stream_));
  }
  map_cap_ = mode_ != MODE_BASIC ? spill_cap_ : map_cap_;
  (void)tree;
  MTC_CUDA(cudaMemcpyAsync(digests_.p, host, sizeof(Digest) * spill_nd_, cudaMemcpyHostToDevice, stream_));
  if (mode_ != MODE_BASIC && spill_cap_) {
    MTC_CUDA(cudaMemcpyAsync(slots_.p, host + sizeof(Digest) * spill_nd_, sizeof(MapSlot) * spill_cap_,
                             cudaMemcpyHostToDevice, stream_));
    // the map's size word lives in device memory too
    set_word_kernel<<<1, 1, 0, stream_>>>(map_size_.p, saved_size);
    note_launch();
    MTC_CUDA(cudaGetLastError());
  }
  map_size_host_ = saved_size;
  return ST_OK;
}

void Engine::release_restart_scratch() {
  if (rs_) {
    destroy_restart_scratch(rs_);  // stream-ordered frees
    rs_ = nullptr;
  }
  restart_stage.release(stream_);
}

uint64_t Engine::device_bytes() const {
  return sizeof(Digest) * digests_.n + labels_.n + rflag_.n +
         sizeof(uint32_t) * (chunk_slot_.n + changed_list_.n + changed_count_.n + map_size_.n + err_.n + fo_list_.n +
                             sh_list_.n + reg_chunk_.n + reg_slot_.n + reg_len_.n + sh_key_.n + sh_prev_.n + hist_.n +
                             rep_.n + rank_.n) +
         sizeof(MapSlot) * slots_.n +
         sizeof(uint64_t) * (fo_val_.n + sort_mat_.n + scan_.n + scan_total_.n + scan2_.n + scan_total2_.n) + stage_.n +
         sizeof(Layout) * lay_.n + sizeof(StepParams) * sp_.n;
}

const uint8_t* Engine::diff_device() const { return stage_.p ? stage_.p + diff_pad_ : nullptr; }

int Engine::copy_diff(void* host, uint64_t cap) {
  if (!stage_.p) return fail(ST_EINVAL, "no checkpoint staged");
  if (cap < diff_len_) return fail(ST_EINVAL, "host buffer too small");
  cudaEvent_t a = ev_[0], b = ev_[1];
  MTC_CUDA(cudaEventRecord(a, stream_));
  MTC_CUDA(cudaMemcpyAsync(host, stage_.p + diff_pad_, diff_len_, cudaMemcpyDeviceToHost, stream_));
  MTC_CUDA(cudaEventRecord(b, stream_));
  MTC_CUDA(cudaEventSynchronize(b));
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  timers[3] = ms * 1e-3;
  return ST_OK;
}

}  // namespace mtc
