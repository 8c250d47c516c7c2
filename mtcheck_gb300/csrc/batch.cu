// batch.cu -- Batch (many engines, one CUDA graph per step) and the autotuner.
#include <algorithm>
#include <cstdlib>
#include <chrono>
#include <map>
#include <mutex>
#include <tuple>

#include "batch.hpp"

namespace mtc {

namespace {
double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}
}  // namespace

namespace {
// MTCHECK_BATCH_LEAF / MTCHECK_BATCH_POOL = 0 or 1 override the defaults
bool env_flag(const char* name, bool dflt) {
  const char* e = std::getenv(name);
  if (!e || !*e) return dflt;
  return e[0] != '0';
}
}  // namespace

Batch::Batch() {
  leaf_batching_ = env_flag("MTCHECK_BATCH_LEAF", leaf_batching_);
  // every member allocates from one stream-ordered pool that keeps what is
  // freed: a batch of many small members otherwise spends its first step in
  // thousands of cudaMalloc calls
  const bool use_pool = env_flag("MTCHECK_BATCH_POOL", true);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  if (use_pool && cudaMemPoolCreate(&pool_, &props) == cudaSuccess) {
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &keep);
  } else {
    pool_ = nullptr;
    cudaGetLastError();
  }
  cudaStreamCreateWithFlags(&origin_, cudaStreamNonBlocking);
  cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&in_, cudaEventDisableTiming);
  cudaEventCreate(&t0_);
  cudaEventCreate(&t1_);
}

Batch::~Batch() {
  if (origin_) cudaStreamSynchronize(origin_);
  for (auto s : streams_) cudaStreamSynchronize(s);
  drop_graph();
  for (auto* e : engs_) delete e;
  for (auto s : streams_) cudaStreamSynchronize(s);
  for (auto s : streams_) cudaStreamDestroy(s);
  if (pool_) cudaMemPoolDestroy(pool_);
  if (members_dev_) cudaFree(members_dev_);
  if (items_dev_) cudaFree(items_dev_);
  if (head_dev_) cudaFree(head_dev_);
  for (auto e : joins_) cudaEventDestroy(e);
  if (fork_) cudaEventDestroy(fork_);
  if (in_) cudaEventDestroy(in_);
  if (t0_) cudaEventDestroy(t0_);
  if (t1_) cudaEventDestroy(t1_);
  if (origin_) cudaStreamDestroy(origin_);
}

int Batch::fail(int code, const std::string& msg) {
  last_error = msg;
  return code;
}

void Batch::drop_parent() {
  if (parent_exec_) cudaGraphExecDestroy(parent_exec_);
  if (parent_) cudaGraphDestroy(parent_);
  parent_exec_ = nullptr;
  parent_ = nullptr;
}

void Batch::drop_graph() {
  drop_parent();
  for (auto& g : pre_)
    if (g) cudaGraphDestroy(g);
  for (auto& g : post_)
    if (g) cudaGraphDestroy(g);
  pre_.assign(engs_.size(), nullptr);
  post_.assign(engs_.size(), nullptr);
  in_kernel_.assign(engs_.size(), 0);
  recs_.assign(engs_.size(), MemberLeaf{});
  sigs_.assign(engs_.size(), 0);
  nodes_.assign(engs_.size(), 0);
  kernels_.assign(engs_.size(), 0);
}

int Batch::add(int mode, int hash_kind, uint32_t chunk_size) {
  cudaStream_t s = nullptr;
  cudaEvent_t j = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return -1;
  if (cudaEventCreateWithFlags(&j, cudaEventDisableTiming) != cudaSuccess) {
    cudaStreamDestroy(s);
    return -1;
  }
  auto* e = new Engine(mode, hash_kind, chunk_size);
  e->set_stream(s);
  e->set_order_after_legacy(true);
  e->set_params_from_host(true);  // the batch's graph replays the member's sequence as captured
  if (pool_) e->set_pool(pool_);
  engs_.push_back(e);
  streams_.push_back(s);
  joins_.push_back(j);
  drop_graph();
  return (int)engs_.size() - 1;
}

#define MTC_BCUDA(call)                                                                              \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return fail(e_ == cudaErrorMemoryAllocation ? ST_ENOMEM : ST_ECUDA,       \
                                       std::string(#call) + ": " + cudaGetErrorString(e_));          \
  } while (0)

int Batch::reserve(const uint64_t* lens, uint64_t* bytes) {
  uint64_t total = 0;
  for (size_t i = 0; i < engs_.size(); i++)
    total += estimate_state_bytes(engs_[i]->mode(), lens[i], engs_[i]->chunk_size());
  if (bytes) *bytes = total;
  if (!pool_) return fail(ST_ENOTSUP, "the batch allocates without a memory pool (MTCHECK_BATCH_POOL=0)");
  void* p = nullptr;
  MTC_BCUDA(cudaMallocFromPoolAsync(&p, total ? total : 1, pool_, origin_));
  MTC_BCUDA(cudaFreeAsync(p, origin_));
  MTC_BCUDA(cudaStreamSynchronize(origin_));
  return ST_OK;
}

// The member's sequence reaches its leaf pass while being captured: when
// its leaves can go through the batched launch, keep its record, close the
// capture there (the part before the leaves) and open the part after it,
// which starts with the partial last chunk, if any, hashed on its own.
int Batch::on_leaves(Engine* e, const LeafArgs& la, cudaStream_t s) {
  MemberLeaf rec;
  if (!leaf_batching_ || !batch_leaf_member(&rec, la)) {
    const cudaError_t ce = e->launch_own_leaves(la, s);
    return ce == cudaSuccess ? ST_OK : ST_ECUDA;
  }
  cudaGraph_t g = nullptr;
  if (cudaStreamEndCapture(s, &g) != cudaSuccess) return ST_ECUDA;
  pre_[cur_] = g;
  recs_[cur_] = rec;
  in_kernel_[cur_] = 1;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) != cudaSuccess) return ST_ECUDA;
  if (la.n_chunks > rec.n_full && launch_leaf_range(la, rec.n_full, la.n_chunks, s) != cudaSuccess) return ST_ECUDA;
  return ST_OK;
}

int Batch::capture_member(size_t i, const uint8_t* data, uint64_t len) {
  for (cudaGraph_t* g : {&pre_[i], &post_[i]}) {
    if (*g) cudaGraphDestroy(*g);
    *g = nullptr;
  }
  in_kernel_[i] = 0;
  const uint64_t l0 = launch_count();
  // the member's graphs become child nodes of the step's graph: captured
  // with plain stream order (no programmatic dependencies)
  PdlSuppress no_pdl;
  cur_ = i;
  engs_[i]->set_leaf_hook(this);
  MTC_BCUDA(cudaStreamBeginCapture(streams_[i], cudaStreamCaptureModeRelaxed));
  int rc = engs_[i]->enqueue(data, len, false);
  engs_[i]->set_leaf_hook(nullptr);
  cudaGraph_t g = nullptr;
  cudaError_t ee = cudaStreamEndCapture(streams_[i], &g);
  if (rc != ST_OK || ee != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    for (cudaGraph_t* p : {&pre_[i], &post_[i]}) {
      if (*p) cudaGraphDestroy(*p);
      *p = nullptr;
    }
    in_kernel_[i] = 0;
    if (rc != ST_OK) return fail(rc, "member " + std::to_string(i) + ": " + engs_[i]->last_error);
    return fail(ST_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ee));
  }
  (in_kernel_[i] ? post_[i] : pre_[i]) = g;
  size_t n = 0, n2 = 0;
  cudaGraphGetNodes(pre_[i], nullptr, &n);
  if (post_[i]) cudaGraphGetNodes(post_[i], nullptr, &n2);
  nodes_[i] = n + n2;
  kernels_[i] = launch_count() - l0;
  sigs_[i] = engs_[i]->signature(data, len);
  stats_.captures++;
  return ST_OK;
}

// The step's graph: the work queue's head is reset and every member's part
// before its leaves runs; then one persistent launch hashes the leaves of
// every member whose record was kept (items (member, tile), largest tiles
// first); then each such member's part after its leaves.
int Batch::build_parent() {
  drop_parent();
  std::vector<uint32_t> order;
  for (uint32_t i = 0; i < engs_.size(); i++)
    if (in_kernel_[i]) order.push_back(i);
  // per-tile cost: bytes per tile, MD5 about twice Murmur3's work per byte
  auto cost = [&](uint32_t i) {
    return (uint64_t)recs_[i].la.cs * (recs_[i].la.hash_kind == HASH_MD5 ? 2 : 1);
  };
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return cost(x) > cost(y); });
  std::vector<uint2> items;
  for (uint32_t i : order) {
    const uint32_t tiles = (recs_[i].n_full + kBatchRows - 1) / kBatchRows;
    for (uint32_t t = 0; t < tiles; t++) items.push_back(make_uint2(i, t));
  }
  if (!order.empty()) {
    if (members_cap_ < engs_.size()) {
      if (members_dev_) cudaFree(members_dev_);
      members_dev_ = nullptr;
      MTC_BCUDA(cudaMalloc(&members_dev_, sizeof(MemberLeaf) * engs_.size()));
      members_cap_ = engs_.size();
    }
    if (items_cap_ < items.size()) {
      if (items_dev_) cudaFree(items_dev_);
      items_dev_ = nullptr;
      MTC_BCUDA(cudaMalloc(&items_dev_, sizeof(uint2) * items.size()));
      items_cap_ = items.size();
    }
    if (!head_dev_) MTC_BCUDA(cudaMalloc(&head_dev_, 256));
    MTC_BCUDA(cudaMemcpy(members_dev_, recs_.data(), sizeof(MemberLeaf) * engs_.size(), cudaMemcpyHostToDevice));
    MTC_BCUDA(cudaMemcpy(items_dev_, items.data(), sizeof(uint2) * items.size(), cudaMemcpyHostToDevice));
  }
  leaf_params_ = BatchLeafParams{members_dev_, items_dev_, (uint32_t)items.size(), 0, head_dev_};
  stats_.batched_leaf_items = items.size();
  stats_.batched_leaf_members = (uint32_t)order.size();

  MTC_BCUDA(cudaGraphCreate(&parent_, 0));
  std::vector<cudaGraphNode_t> before;  // what the batched launch waits for
  if (!order.empty()) {
    cudaMemsetParams mp{};
    mp.dst = head_dev_;
    mp.value = 0;
    mp.elementSize = 4;
    mp.width = 1;
    mp.height = 1;
    cudaGraphNode_t reset = nullptr;
    MTC_BCUDA(cudaGraphAddMemsetNode(&reset, parent_, nullptr, 0, &mp));
    before.push_back(reset);
  }
  for (size_t i = 0; i < engs_.size(); i++) {
    cudaGraphNode_t a = nullptr;
    MTC_BCUDA(cudaGraphAddChildGraphNode(&a, parent_, nullptr, 0, pre_[i]));
    if (in_kernel_[i]) before.push_back(a);
  }
  if (!order.empty()) {
    cudaKernelNodeParams kp{};
    void* args[1];
    MTC_BCUDA(batch_leaf_node_params(leaf_params_, &kp, args));
    cudaGraphNode_t k = nullptr;
    MTC_BCUDA(cudaGraphAddKernelNode(&k, parent_, before.data(), before.size(), &kp));
    for (size_t i = 0; i < engs_.size(); i++) {
      if (!in_kernel_[i]) continue;
      cudaGraphNode_t b = nullptr;
      MTC_BCUDA(cudaGraphAddChildGraphNode(&b, parent_, &k, 1, post_[i]));
    }
  }
  cudaError_t ie = cudaGraphInstantiate(&parent_exec_, parent_, 0);
  if (ie != cudaSuccess) {
    parent_exec_ = nullptr;
    drop_parent();
    return fail(ST_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
  }
  return ST_OK;
}

int Batch::checkpoint(const uint8_t* const* data, const uint64_t* lens, bool make_baseline, uint64_t* diff_lens) {
  const double t_call = now_ms();
  if (engs_.empty()) return fail(ST_EINVAL, "empty batch");
  if (!data || !lens) return fail(ST_EINVAL, "NULL argument");
  // 1. allocations, validation, map growth: outside any capture
  bool any_fresh = false;
  for (size_t i = 0; i < engs_.size(); i++) {
    int rc = engs_[i]->prepare(data[i], lens[i], make_baseline, headroom_);
    if (rc) return fail(rc, "member " + std::to_string(i) + ": " + engs_[i]->last_error);
    any_fresh = any_fresh || engs_[i]->fresh();
  }
  // prepare's own stream work (map rehash) is ordered before the step on
  // each member's stream; nothing waits for it here
  const double t_prep = now_ms();
  const bool graph = use_graph_ && !any_fresh;
  // 2. (re)capture the members whose device buffers moved; their streams
  // (allocations, rehash) and those of members whose prepare issued other
  // work are joined into the origin stream before the step
  std::vector<char> join(engs_.size(), 0);
  if (graph) {
    bool rebuild = !parent_exec_;
    for (size_t i = 0; i < engs_.size(); i++) {
      if (engs_[i]->take_stream_work()) join[i] = 1;
      if (!pre_[i] || sigs_[i] != engs_[i]->signature(data[i], lens[i])) {
        int rc = capture_member(i, data[i], lens[i]);
        if (rc) return rc;
        join[i] = 1;
        rebuild = true;  // moved buffers: new records and graphs
      }
    }
    if (rebuild) {
      int rc = build_parent();
      if (rc) return rc;
    }
  }
  // 3. issue: the step starts after the work already on the legacy default
  // stream (where the inputs are usually written): one launch of the parent
  // graph on the origin stream, or every member on its own stream between a
  // fork and a join on the origin stream
  const double t_cap = now_ms();
  const uint64_t l0 = launch_count();
  MTC_BCUDA(cudaEventRecord(in_, cudaStreamLegacy));
  MTC_BCUDA(cudaStreamWaitEvent(origin_, in_, 0));
  uint64_t nodes = 0, kernels = 0;
  if (graph) {
    for (size_t i = 0; i < engs_.size(); i++) {
      if (join[i]) {
        MTC_BCUDA(cudaEventRecord(joins_[i], streams_[i]));
        MTC_BCUDA(cudaStreamWaitEvent(origin_, joins_[i], 0));
      }
      engs_[i]->stage_params();
      nodes += nodes_[i];
      kernels += kernels_[i];
    }
    if (stats_.batched_leaf_members) kernels += 1;  // the batched leaf launch
    MTC_BCUDA(cudaEventRecord(t0_, origin_));
    MTC_BCUDA(cudaGraphLaunch(parent_exec_, origin_));
  } else {
    MTC_BCUDA(cudaEventRecord(t0_, origin_));
    MTC_BCUDA(cudaEventRecord(fork_, origin_));
    for (size_t i = 0; i < engs_.size(); i++) {
      MTC_BCUDA(cudaStreamWaitEvent(streams_[i], fork_, 0));
      engs_[i]->stage_params();
      int rc = engs_[i]->enqueue(data[i], lens[i], false);
      if (rc) return fail(rc, "member " + std::to_string(i) + ": " + engs_[i]->last_error);
      MTC_BCUDA(cudaEventRecord(joins_[i], streams_[i]));
      MTC_BCUDA(cudaStreamWaitEvent(origin_, joins_[i], 0));
    }
  }
  MTC_BCUDA(cudaEventRecord(t1_, origin_));
  if (graph) {
    note_launch((uint32_t)kernels);
    stats_.graph_nodes = nodes;
    stats_.kernels_per_step = kernels;
  } else {
    stats_.kernels_per_step = launch_count() - l0;
  }
  stats_.last_used_graph = graph ? 1 : 0;
  const double t_issue = now_ms();
  MTC_BCUDA(cudaEventSynchronize(t1_));
  const double t_wait = now_ms();
  float ms = 0;
  cudaEventElapsedTime(&ms, t0_, t1_);
  stats_.last_device_ms = ms;
  // 4. per-member completion, then advance like checkpoint(data, len, diff_h, make_baseline)
  for (size_t i = 0; i < engs_.size(); i++) {
    engs_[i]->release_retired();
    int rc = engs_[i]->complete(lens[i], nullptr);
    if (rc) return fail(rc, "member " + std::to_string(i) + ": " + engs_[i]->last_error);
    if (diff_lens) diff_lens[i] = engs_[i]->diff_len();
  }
  for (auto* e : engs_) e->current_id += 1;
  stats_.steps++;
  const double t_end = now_ms();
  stats_.last_call_ms = t_end - t_call;
  stats_.host_ms[0] = t_prep - t_call;
  stats_.host_ms[1] = t_cap - t_prep;
  stats_.host_ms[2] = t_issue - t_cap;
  stats_.host_ms[3] = t_wait - t_issue;
  stats_.host_ms[4] = t_end - t_wait;
  return ST_OK;
}

// ---------------------------------------------------------------------------
// Autotuner
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  // SplitMix64 finaliser (Steele, Lea, Flood 2014)
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__global__ void tune_fill_kernel(uint8_t* p, uint64_t len, uint64_t seed) {
  const uint64_t words = len / 8;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x)
    reinterpret_cast<uint64_t*>(p)[i] = mix64(seed + i);
  if (blockIdx.x == 0 && threadIdx.x < (len & 7)) p[words * 8 + threadIdx.x] = (uint8_t)mix64(seed ^ threadIdx.x);
}

// Rewrite the first word of about 1/stride of the chunks.
__global__ void tune_touch_kernel(uint8_t* p, uint64_t len, uint32_t cs, uint32_t stride, uint64_t seed) {
  const uint64_t n = len / cs;
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x)
    if (mix64(seed + c) % stride == 0) p[c * cs] ^= (uint8_t)(1 + (mix64(c ^ seed) & 0x7f));
}

std::mutex g_tune_mu;
std::map<std::tuple<int, int, uint32_t, int>, TuneResult> g_tune_cache;

int log2_bucket(uint64_t len) {
  int b = 0;
  while ((1ull << (b + 1)) <= len) b++;
  return b;
}

}  // namespace

int autotune(int mode, int hash_kind, uint32_t chunk_size, uint64_t len, bool use_cache, TuneResult* out,
             std::string* err) {
  const auto key = std::make_tuple(mode, hash_kind, chunk_size, log2_bucket(len));
  if (use_cache) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      *out = it->second;
      return ST_OK;
    }
  }
  if (mode == MODE_FULL) {  // a device-to-device copy: nothing to tune
    *out = TuneResult{};
    return ST_OK;
  }
  uint8_t* buf = nullptr;
  if (cudaMalloc(&buf, len) != cudaSuccess) {
    if (err) *err = "autotune: cannot allocate the sample buffer";
    return ST_ENOMEM;
  }
  cudaStream_t s = nullptr;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const uint32_t grid = (uint32_t)num_sms() * 8;

  struct Cand {
    LeafTune t;
    double load;
  };
  std::vector<Cand> cands;
  cands.push_back({default_leaf_tune(hash_kind), 0.75});  // the default shape first
  const double loads_tree[] = {0.5, 0.75, 0.9};
  const bool has_map = mode != MODE_BASIC && mode != MODE_FULL;
  for (int rows : {256, 128})
    for (int per_sm : {1, 2, 3, 4}) cands.push_back({LeafTune{rows, per_sm, 0}, 0.75});
  cands.push_back({LeafTune{256, 0, 1}, 0.75});
  // a warp per chunk (large chunks only: below 1 KiB a warp would spend its
  // loads on a few hundred bytes)
  if (chunk_size >= 1024 && chunk_size <= 4096) cands.push_back({LeafTune{256, 0, 1, 32}, 0.75});
  if (has_map)
    for (double l : loads_tree)
      if (l != 0.75) cands.push_back({LeafTune{256, 0, 0}, l});

  TuneResult best;
  best.ms = 1e30;
  int rc = ST_OK;
  const int kSteps = 3;
  for (size_t ci = 0; ci < cands.size() && rc == ST_OK; ci++) {
    Engine e(mode, hash_kind, chunk_size);
    e.set_stream(s);
    e.set_leaf_tune(cands[ci].t);
    e.set_max_load(cands[ci].load);
    tune_fill_kernel<<<grid, 256, 0, s>>>(buf, len, 0x5eed);
    HeaderHost h;
    rc = e.checkpoint(buf, len, true, &h);
    if (rc) break;
    e.current_id++;
    // one untimed incremental step: captures the replayed launch sequence
    tune_touch_kernel<<<grid, 256, 0, s>>>(buf, len, chunk_size, 50, 0x0fff);
    rc = e.checkpoint(buf, len, false, &h);
    if (rc) break;
    e.current_id++;
    double sum = 0;
    for (int st = 0; st < kSteps; st++) {
      tune_touch_kernel<<<grid, 256, 0, s>>>(buf, len, chunk_size, 50, 0x1000 + st);
      cudaEventRecord(a, s);
      rc = e.checkpoint(buf, len, false, &h);
      cudaEventRecord(b, s);
      if (rc) break;
      cudaEventSynchronize(b);
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      sum += ms;
      e.current_id++;
    }
    if (rc) break;
    const double mean = sum / kSteps;
    if (ci == 0) best.default_ms = mean;  // first candidate: the default shape
    if (mean < best.ms) {
      best.ms = mean;
      best.leaf = cands[ci].t;
      best.max_load = cands[ci].load;
    }
  }
  best.candidates = (int)cands.size();
  cudaStreamSynchronize(s);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaStreamDestroy(s);
  cudaFree(buf);
  if (rc) {
    if (err) *err = "autotune: a trial checkpoint failed";
    return rc;
  }
  *out = best;
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tune_cache[key] = best;
  return ST_OK;
}

}  // namespace mtc
