// server.cu -- the request-serving loop (see server.hpp).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <set>

#include <sys/mman.h>
#include <unistd.h>

#include "server.hpp"

namespace mtc {

// diff bytes the worker copies out ahead of need in one pass of its loop,
// and at most in flight on the copy engine from those passes: a deeper
// queue of copies makes every other copy of the process (an archive, a
// caller's read-back) wait behind it
constexpr uint64_t kSpillStepBytes = 64ull << 20;
constexpr uint64_t kSpillInFlightBytes = 512ull << 20;

// Device-to-device copy of an archived diff by the SMs rather than a copy
// engine (which the spills keep busy).  Sources are 4-byte aligned (a diff
// starts at its staging buffer's pad, a multiple of 4), destinations are
// pool allocations.
__global__ void archive_copy_kernel(uint8_t* __restrict__ dst, const uint8_t* __restrict__ src, uint64_t n) {
  const uint64_t words = n / 4;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint32_t* s4 = reinterpret_cast<const uint32_t*>(src);
  uint32_t* d4 = reinterpret_cast<uint32_t*>(dst);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += stride) d4[i] = s4[i];
  const uint64_t t = words * 4 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n && t < words * 4 + 4) dst[t] = src[t];
}
static cudaError_t archive_copy(uint8_t* dst, const uint8_t* src, uint64_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if ((reinterpret_cast<uintptr_t>(src) & 3) || (reinterpret_cast<uintptr_t>(dst) & 3))
    return cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToDevice, s);
  const uint64_t words = n / 4 + 1;
  const uint64_t blocks = std::min<uint64_t>((words + 255) / 256, 1024);
  archive_copy_kernel<<<(unsigned)blocks, 256, 0, s>>>(dst, src, n);
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// PinnedArena
// ---------------------------------------------------------------------------
PinnedArena::~PinnedArena() {
  {
    std::lock_guard<std::mutex> g(mu_);
    stop_ = true;
  }
  cv_.notify_all();
  if (helper_.joinable()) helper_.join();
  for (const auto& m : all_) {
    cudaHostUnregister(m.first);
    munmap(m.first, m.second);
  }
}

uint64_t PinnedArena::cls(uint64_t n) {
  constexpr uint64_t kMin = 64ull << 10;
  if (n <= kMin) return kMin;
  uint64_t p = kMin;
  while (p * 2 <= n) p <<= 1;  // p <= n < 2p
  const uint64_t q = p / 4;
  return (n + q - 1) / q * q;
}

bool PinnedArena::add_slab(uint64_t bytes) {
  // Map and touch the pages first, then register them: cudaHostAlloc holds
  // the driver for the whole time it takes (about 75 ms per GiB), during
  // which every CUDA call of every other thread waits; registering pages
  // already present takes about 2 ms per GiB.
  void* q = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (q == MAP_FAILED) return false;
  const long page = sysconf(_SC_PAGESIZE);
  const uint64_t step = page > 0 ? (uint64_t)page : 4096;
  for (uint64_t o = 0; o < bytes; o += step) static_cast<volatile uint8_t*>(q)[o] = 0;
  if (cudaHostRegister(q, bytes, cudaHostRegisterDefault) != cudaSuccess) {
    cudaGetLastError();
    munmap(q, bytes);
    return false;
  }
  std::lock_guard<std::mutex> g(mu_);
  all_.emplace_back(static_cast<uint8_t*>(q), bytes);
  slabs_.push_back({static_cast<uint8_t*>(q), bytes});
  reserved_ += bytes;
  spare_ += bytes;
  return true;
}

bool PinnedArena::reserve(uint64_t bytes) {
  constexpr uint64_t kGiB = 1ull << 30, kMin = 256ull << 20;
  while (reserved() < bytes) {
    const uint64_t left = bytes - reserved();
    const uint64_t slab = left < kMin ? kMin : (left < kGiB ? left : kGiB);
    if (!add_slab(slab)) return false;
  }
  return true;
}

void PinnedArena::keep_spare(int device, uint64_t bytes) {
  std::lock_guard<std::mutex> g(mu_);
  spare_target_ = bytes;
  if (!helper_.joinable() && bytes) helper_ = std::thread([this, device] { helper(device); });
}

void PinnedArena::helper(int device) {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> g(mu_);
  while (!stop_) {
    cv_.wait(g, [&] { return stop_ || spare_ < spare_target_; });
    if (stop_) break;
    g.unlock();
    const bool ok = add_slab(1ull << 30);
    g.lock();
    if (!ok) spare_target_ = 0;  // host memory exhausted: stop trying
  }
}

uint64_t PinnedArena::reserved() {
  std::lock_guard<std::mutex> g(mu_);
  return reserved_;
}

uint64_t PinnedArena::sync_grows() {
  std::lock_guard<std::mutex> g(mu_);
  return sync_grows_;
}

uint8_t* PinnedArena::carve(uint64_t c) {
  for (Slab& sl : slabs_)
    if (sl.left >= c) {
      uint8_t* p = sl.next;
      sl.next += c;
      sl.left -= c;
      spare_ -= c;
      return p;
    }
  return nullptr;
}

uint8_t* PinnedArena::alloc(uint64_t n) {
  const uint64_t c = cls(n);
  {
    std::lock_guard<std::mutex> g(mu_);
    auto& fl = free_[c];
    if (!fl.empty()) {
      uint8_t* p = fl.back();
      fl.pop_back();
      return p;
    }
    uint8_t* p = carve(c);
    if (spare_ < spare_target_) cv_.notify_one();
    if (p) return p;
    sync_grows_++;
  }
  if (!add_slab(std::max<uint64_t>(c, 256ull << 20))) return nullptr;
  std::lock_guard<std::mutex> g(mu_);
  return carve(c);
}

void PinnedArena::free(uint8_t* p, uint64_t n) {
  if (!p) return;
  std::lock_guard<std::mutex> g(mu_);
  free_[cls(n)].push_back(p);
}

// ---------------------------------------------------------------------------
// Server
// ---------------------------------------------------------------------------
double Server::now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

Server::Server(const ServerOptions& o) : opt_(o) {
  if (opt_.max_inflight == 0) opt_.max_inflight = 1;
  if (opt_.id_headroom == 0) opt_.id_headroom = 1;
  cudaGetDevice(&device_);
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device_;
  if (cudaMemPoolCreate(&pool_, &props) == cudaSuccess) {
    // keep freed memory in the pool: returning it to the driver would
    // synchronise at every stream synchronisation point
    uint64_t keep = std::numeric_limits<uint64_t>::max();
    cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &keep);
  } else {
    pool_ = nullptr;
    cudaGetLastError();
  }
  if (pool_ && opt_.reserve_hbm) {
    // grow the pool to the budget once; freed memory stays in the pool
    cudaStream_t s = nullptr;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    void* p = nullptr;
    // the budget and an eighth more: staged restart inputs and the pool's
    // fragmentation are outside the budget's accounting, and growing the
    // pool while requests run maps memory under the driver's lock
    if (cudaMallocFromPoolAsync(&p, opt_.hbm_budget + opt_.hbm_budget / 8, pool_, s) == cudaSuccess)
      cudaFreeAsync(p, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    cudaGetLastError();
  }
  cudaStreamCreateWithFlags(&spill_s_, cudaStreamNonBlocking);
  if (opt_.pinned_reserve) arena_.reserve(opt_.pinned_reserve);
  // with a reserve, a helper thread keeps an eighth of it pinned ahead of
  // the spills
  if (opt_.pinned_reserve) arena_.keep_spare(device_, opt_.pinned_reserve / 8);
  thread_ = std::thread([this] { worker(); });
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> g(mu_);
    stop_ = true;
  }
  cv_work_.notify_all();
  if (thread_.joinable()) thread_.join();
  if (spill_s_) {
    cudaStreamSynchronize(spill_s_);
    cudaStreamDestroy(spill_s_);
  }
  for (const SpillBatch& sb : spills_) events_.push_back(sb.ev);
  spills_.clear();
  for (auto& pp : procs_) {
    Proc& p = *pp;
    cudaStreamSynchronize(p.s);
    if (p.exec) cudaGraphExecDestroy(p.exec);
    for (auto& a : p.chain)
      if (a.dev) cudaFreeAsync(a.dev, p.s);
    p.eng.reset();  // stream-ordered frees on p.s
    cudaStreamSynchronize(p.s);
    cudaStreamDestroy(p.s);
  }
  procs_.clear();
  for (auto e : events_) cudaEventDestroy(e);
  cudaDeviceSynchronize();
  if (pool_) cudaMemPoolDestroy(pool_);
}

void Server::set_error(const std::string& e) {
  std::lock_guard<std::mutex> g(mu_);
  err_ = e;
}

std::string Server::error() {
  std::lock_guard<std::mutex> g(mu_);
  return err_;
}

cudaEvent_t Server::get_event() {
  // caller holds mu_
  if (!events_.empty()) {
    cudaEvent_t e = events_.back();
    events_.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  return e;
}

void Server::put_event(cudaEvent_t e) {
  std::lock_guard<std::mutex> g(mu_);
  events_.push_back(e);
}

int Server::add_process(int mode, int hash_kind, uint32_t chunk_size, uint32_t* pid) {
  if (!pool_) {
    set_error("no stream-ordered memory pool on this device");
    return ST_ENOTSUP;
  }
  auto p = std::make_unique<Proc>();
  if (cudaStreamCreateWithFlags(&p->s, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cannot create a stream");
    return ST_ECUDA;
  }
  p->eng = std::make_unique<Engine>(mode, hash_kind, chunk_size);
  p->eng->set_stream(p->s);
  p->eng->set_pool(pool_);
  p->eng->set_params_from_host(true);  // its captured graphs replay as captured
  std::lock_guard<std::mutex> g(mu_);
  procs_.push_back(std::move(p));
  *pid = (uint32_t)procs_.size() - 1;
  return ST_OK;
}

int Server::submit_checkpoint(uint32_t pid, const uint8_t* data, uint64_t len, bool make_baseline, uint64_t* ticket) {
  if (!data || len == 0) {
    set_error("empty buffer");
    return ST_EINVAL;
  }
  std::unique_lock<std::mutex> g(mu_);
  if (pid >= procs_.size()) {
    err_ = "unknown process";
    return ST_EINVAL;
  }
  if (stop_) return ST_EINVAL;
  Req r{next_ticket_++, pid, REQ_CHECKPOINT, data, nullptr, len, make_baseline, 0, now_ms(), get_event()};
  // the buffer is complete once the work already on the legacy default
  // stream (where the caller wrote it) has run
  cudaEventRecord(r.ready, cudaStreamLegacy);
  inbox_.push_back(r);
  outstanding_++;
  st_.submitted++;
  if (ticket) *ticket = r.ticket;
  g.unlock();
  cv_work_.notify_one();
  return ST_OK;
}

int Server::submit_restart(uint32_t pid, uint32_t chkpt_id, uint8_t* out, uint64_t len, uint64_t* ticket) {
  if (!out || len == 0) {
    set_error("empty output buffer");
    return ST_EINVAL;
  }
  std::unique_lock<std::mutex> g(mu_);
  if (pid >= procs_.size()) {
    err_ = "unknown process";
    return ST_EINVAL;
  }
  if (stop_) return ST_EINVAL;
  Req r{next_ticket_++, pid, REQ_RESTART, nullptr, out, len, false, chkpt_id, now_ms(), get_event()};
  cudaEventRecord(r.ready, cudaStreamLegacy);
  inbox_.push_back(r);
  outstanding_++;
  st_.submitted++;
  if (ticket) *ticket = r.ticket;
  g.unlock();
  cv_work_.notify_one();
  return ST_OK;
}

uint32_t Server::poll(Completion* out, uint32_t max, double wait_ms) {
  std::unique_lock<std::mutex> g(mu_);
  if (done_.empty() && wait_ms > 0)
    cv_done_.wait_for(g, std::chrono::microseconds((int64_t)(wait_ms * 1000)), [&] { return !done_.empty(); });
  uint32_t n = 0;
  while (n < max && !done_.empty()) {
    out[n++] = done_.front();
    done_.pop_front();
  }
  return n;
}

bool Server::drain(double timeout_ms) {
  std::unique_lock<std::mutex> g(mu_);
  return cv_done_.wait_for(g, std::chrono::microseconds((int64_t)(timeout_ms * 1000)),
                           [&] { return outstanding_ == 0; });
}

int Server::chain_length(uint32_t pid, uint32_t* n) {
  std::lock_guard<std::mutex> g(mu_);
  if (pid >= procs_.size()) return ST_EINVAL;
  *n = (uint32_t)procs_[pid]->chain.size();
  return ST_OK;
}

int Server::copy_diff(uint32_t pid, uint32_t id, void* host, uint64_t cap, uint64_t* len) {
  std::lock_guard<std::mutex> g(mu_);
  if (pid >= procs_.size()) return ST_EINVAL;
  Proc& p = *procs_[pid];
  if (id >= p.chain.size()) return ST_EINVAL;
  Archived& a = p.chain[id];
  if (len) *len = a.len;
  if (!host) return ST_OK;
  if (cap < a.len) return ST_EINVAL;
  // the archive copy and any spill of this entry run on the process's stream
  if (cudaStreamSynchronize(p.s) != cudaSuccess) return ST_ECUDA;
  if (a.dev) {
    if (cudaMemcpy(host, a.dev, a.len, cudaMemcpyDeviceToHost) != cudaSuccess) return ST_ECUDA;
  } else {
    std::memcpy(host, a.host, a.len);
  }
  return ST_OK;
}

ServerStats Server::stats() {
  std::lock_guard<std::mutex> g(mu_);
  ServerStats s = st_;
  s.pinned_reserved = arena_.reserved();
  s.pinned_sync_grows = arena_.sync_grows();
  if (pool_) {
    cuuint64_t v = 0;
    if (cudaMemPoolGetAttribute(pool_, cudaMemPoolAttrReservedMemHigh, &v) == cudaSuccess) s.pool_reserved_high = v;
    if (cudaMemPoolGetAttribute(pool_, cudaMemPoolAttrUsedMemHigh, &v) == cudaSuccess) s.pool_used_high = v;
    cudaGetLastError();
  }
  return s;
}

void Server::push_completion(const Completion& c) {
  {
    std::lock_guard<std::mutex> g(mu_);
    done_.push_back(c);
    outstanding_--;
    st_.completed++;
    if (c.status != ST_OK) st_.failed++;
  }
  cv_done_.notify_all();
}

// ---- memory accounting -----------------------------------------------------
uint64_t Server::need_bytes(const Req& r, const Proc& p) const {
  const Engine& e = *p.eng;
  const uint64_t N = (r.len + e.chunk_size() - 1) / e.chunk_size();
  uint64_t need = 0;
  if (e.spilled()) need += p.spill_len + estimate_state_bytes(e.mode(), r.len, e.chunk_size()) / 2;
  if (r.kind == REQ_CHECKPOINT) {
    if (p.state_dev == 0 && !e.spilled()) need += estimate_state_bytes(e.mode(), r.len, e.chunk_size());
    // the archived diff: the worst case is the whole buffer (a baseline);
    // afterwards twice the latest size, at least 1/16 of the buffer -- a
    // larger diff overshoots the budget until the next admission spills
    const uint64_t worst = 32 + 12 * (N + 1) + (N + 1) * e.chunk_size();
    need += p.chain.empty() ? worst : std::min(worst, std::max(2 * p.last_diff, r.len / 16));
  } else {
    for (uint32_t k = 0; k <= r.chkpt_id && k < p.chain.size(); k++)
      if (!p.chain[k].dev) need += p.chain[k].len;  // staged back for the restart
    need += N * 96 + (uint64_t)(r.chkpt_id + 1) * (N + 1) * 16;  // restart scratch (64-bit table cells)
  }
  return need;
}

void Server::refresh_state_bytes(Proc& p) {
  p.state_dev = p.eng->spilled() ? 0 : p.eng->device_bytes();
  p.scratch_dev = p.eng->restart_scratch_bytes();
}

uint64_t Server::used_bytes() const {
  uint64_t u = chain_dev_;
  for (const Proc* pp : view_) u += pp->state_dev + pp->scratch_dev;
  return u;
}

void Server::reap_spills() {
  for (size_t b = 0; b < spills_.size();) {
    SpillBatch& sb = spills_[b];
    if (cudaEventQuery(sb.ev) == cudaErrorNotReady) {
      b++;
      continue;
    }
    for (size_t i = 0; i < sb.items.size();) {
      Proc& p = *view_[sb.items[i].first];
      // a running restart of the process may read the device copy
      if (p.busy) {
        i++;
        continue;
      }
      {
        // under the lock: copy_diff reads the device copy while it holds it
        std::lock_guard<std::mutex> g(mu_);
        Archived& a = p.chain[sb.items[i].second];
        cudaFreeAsync(a.dev, p.s);
        a.dev = nullptr;
        a.spilling = false;
        chain_dev_ -= a.len;
        p.chain_dev -= a.len;
        p.chain_moving -= a.len;
        spilling_bytes_ -= a.len;
      }
      sb.items[i] = sb.items.back();
      sb.items.pop_back();
    }
    if (sb.items.empty()) {
      put_event(sb.ev);
      spills_.erase(spills_.begin() + (long)b);
    } else {
      b++;
    }
  }
}

uint64_t Server::spill_chains(uint64_t target, uint32_t except, uint64_t max_bytes) {
  SpillBatch sb{nullptr, {}};
  uint64_t issued = 0;
  bool out_of_pinned = false;
  while (!out_of_pinned && issued < max_bytes && used_bytes() - spilling_bytes_ > target) {
    // the oldest resident archived checkpoints of the least recently used idle process
    Proc* victim = nullptr;
    uint32_t vid = 0;
    for (uint32_t i = 0; i < view_.size(); i++) {
      Proc& p = *view_[i];
      if (p.busy || i == except || p.chain_dev == p.chain_moving) continue;
      if (!victim || p.lru < victim->lru) {
        victim = &p;
        vid = i;
      }
    }
    if (!victim) break;
    {
      // the spill stream copies after the archive copies on the process's stream
      cudaEvent_t ev;
      {
        std::lock_guard<std::mutex> g(mu_);
        ev = get_event();
      }
      cudaEventRecord(ev, victim->s);
      cudaStreamWaitEvent(spill_s_, ev, 0);
      put_event(ev);
    }
    for (uint32_t k = 0; k < victim->chain.size() && issued < max_bytes; k++) {
      Archived& a = victim->chain[k];
      if (!a.dev || a.spilling) continue;
      uint8_t* h = arena_.alloc(a.len);
      if (!h) {
        out_of_pinned = true;
        break;
      }
      cudaMemcpyAsync(h, a.dev, a.len, cudaMemcpyDeviceToHost, spill_s_);
      std::lock_guard<std::mutex> g(mu_);
      a.host = h;
      a.spilling = true;
      sb.items.emplace_back(vid, k);
      spilling_bytes_ += a.len;
      victim->chain_moving += a.len;
      st_.spilled_diffs++;
      st_.spilled_bytes += a.len;
      issued += a.len;
    }
  }
  if (!sb.items.empty()) {
    {
      std::lock_guard<std::mutex> g(mu_);
      sb.ev = get_event();
    }
    cudaEventRecord(sb.ev, spill_s_);
    spills_.push_back(std::move(sb));
  }
  return issued;
}

void Server::spill_state(Proc& p) {
  const uint64_t n = p.eng->spill_bytes();
  uint8_t* h = arena_.alloc(n);
  if (!h) return;
  if (p.eng->spill_to_host(h) != ST_OK) {
    arena_.free(h, n);
    return;
  }
  p.spill = h;
  p.spill_len = n;
  if (p.exec) {
    cudaGraphExecDestroy(p.exec);
    p.exec = nullptr;
  }
  refresh_state_bytes(p);
  std::lock_guard<std::mutex> g(mu_);
  st_.spilled_states++;
  st_.spilled_bytes += n;
}

int Server::restore_state(Proc& p) {
  int rc = p.eng->restore_from_host(p.spill);
  if (rc) return rc;
  // the pinned copy is read by the stream; it returns to the arena when the
  // request that restored it completes
  refresh_state_bytes(p);
  std::lock_guard<std::mutex> g(mu_);
  st_.restored_states++;
  return ST_OK;
}

uint64_t Server::drop_scratch(uint64_t target, uint32_t except) {
  // the restart tables of the least recently used idle processes (a cache:
  // dropping them costs only the next restart's allocation)
  uint64_t dropped = 0;
  while (used_bytes() > target) {
    Proc* victim = nullptr;
    for (uint32_t i = 0; i < view_.size(); i++) {
      Proc& p = *view_[i];
      if (p.busy || i == except || p.scratch_dev == 0) continue;
      if (!victim || p.lru < victim->lru) victim = &p;
    }
    if (!victim) break;
    dropped += victim->scratch_dev;
    victim->eng->release_restart_scratch();
    victim->scratch_dev = 0;
  }
  return dropped;
}

bool Server::make_room(uint64_t need, uint32_t except) {
  // free down to 95% of the budget, so that the next admissions find room
  const uint64_t target = opt_.hbm_budget - opt_.hbm_budget / 20;
  // 0. restart tables
  drop_scratch(need >= target ? 0 : target - need, except);
  if (used_bytes() + need <= target) return true;
  // 1. archived checkpoints, copied to pinned memory on their processes'
  //    streams; the request is admitted once enough of the copies have landed
  spill_chains(need >= target ? 0 : target - need, except, std::numeric_limits<uint64_t>::max());
  if (used_bytes() + need <= opt_.hbm_budget) return true;
  if (used_bytes() - spilling_bytes_ + need <= opt_.hbm_budget) return false;
  // 2. the digest state of the least recently used idle process
  while (used_bytes() - spilling_bytes_ + need > target) {
    Proc* victim = nullptr;
    for (uint32_t i = 0; i < view_.size(); i++) {
      Proc& p = *view_[i];
      if (p.busy || i == except || p.state_dev == 0 || p.eng->mode() == MODE_FULL) continue;
      if (!victim || p.lru < victim->lru) victim = &p;
    }
    if (!victim) break;
    const uint64_t before = victim->state_dev;
    spill_state(*victim);
    if (victim->state_dev == before) break;  // no pinned memory left
  }
  return used_bytes() + need <= opt_.hbm_budget;
}

// ---- request execution -------------------------------------------------------
int Server::ensure_graph(Proc& p, const uint8_t* data, uint64_t len) {
  Engine& e = *p.eng;
  const uint64_t sig = e.signature(data, len);
  if (p.exec && p.sig == sig) return ST_OK;
  if (p.exec) cudaGraphExecDestroy(p.exec);
  p.exec = nullptr;
  if (cudaStreamBeginCapture(p.s, cudaStreamCaptureModeRelaxed) != cudaSuccess) return ST_ECUDA;
  int rc = e.enqueue(data, len, false);
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamEndCapture(p.s, &g);
  if (rc || ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return rc ? rc : ST_ECUDA;
  }
  ce = cudaGraphInstantiate(&p.exec, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) {
    p.exec = nullptr;
    return ST_ECUDA;
  }
  p.sig = sig;
  std::lock_guard<std::mutex> lk(mu_);
  st_.graph_captures++;
  return ST_OK;
}

int Server::start_checkpoint(Req& r, Proc& p) {
  Engine& e = *p.eng;
  bool restored = false;
  if (e.spilled()) {
    int rc = restore_state(p);
    if (rc) return rc;
    restored = true;
  }
  if (cudaStreamWaitEvent(p.s, r.ready, 0) != cudaSuccess) return ST_ECUDA;
  StepTimer st_ck("checkpoint start", r.pid);
  int rc = e.prepare(r.data, r.len, r.make_baseline, opt_.id_headroom);
  if (rc) return rc;
  // a restored state has new device addresses: issuing it once costs less
  // than capturing a graph that the next eviction may throw away
  const bool graph = opt_.use_graph && !e.fresh() && !restored;
  if (graph) {
    rc = ensure_graph(p, r.data, r.len);
    if (rc) return rc;
    e.stage_params();
    if (cudaGraphLaunch(p.exec, p.s) != cudaSuccess) return ST_ECUDA;
    std::lock_guard<std::mutex> lk(mu_);
    st_.graph_replays++;
  } else {
    if (e.mode() != MODE_FULL) e.stage_params();
    rc = e.enqueue(r.data, r.len, false);
    if (rc) return rc;
  }
  return ST_OK;
}

int Server::start_restart(Req& r, Proc& p, std::vector<uint8_t*>* temps) {
  Engine& e = *p.eng;
  if (r.chkpt_id >= p.chain.size()) return ST_EINVAL;
  if (e.spilled()) {
    int rc = restore_state(p);
    if (rc) return rc;
  }
  StepTimer st_all("restart start", r.pid);
  const size_t n = p.chain.size();
  std::vector<const uint8_t*> ptrs(n, nullptr);
  std::vector<uint64_t> lens(n, 0);
  std::vector<HeaderHost> hdrs(n);
  for (size_t k = 0; k < n; k++) {
    Archived& a = p.chain[k];
    lens[k] = a.len;
    hdrs[k] = a.hdr;
    if (k > r.chkpt_id) continue;
    if (a.dev) {
      ptrs[k] = a.dev;
    } else {
      // a spilled checkpoint comes back for this restart only
      uint8_t* t = nullptr;
      if (cudaMallocFromPoolAsync(reinterpret_cast<void**>(&t), a.len ? a.len : 1, pool_, p.s) != cudaSuccess)
        return ST_ENOMEM;
      cudaMemcpyAsync(t, a.host, a.len, cudaMemcpyHostToDevice, p.s);
      temps->push_back(t);
      ptrs[k] = t;
      std::lock_guard<std::mutex> lk(mu_);
      st_.staged_diffs++;
    }
  }
  if (cudaStreamWaitEvent(p.s, r.ready, 0) != cudaSuccess) return ST_ECUDA;
  StepTimer st_enq("restart_enqueue", r.pid);
  int rc = e.restart_enqueue(r.out, r.len, ptrs, lens, hdrs, r.chkpt_id);
  for (uint8_t* t : *temps) cudaFreeAsync(t, p.s);  // after the restart, in stream order
  return rc;
}

bool Server::try_start(Req& r) {
  Proc& p = *view_[r.pid];
  const uint64_t need = need_bytes(r, p);
  const double t_room = now_ms();
  const bool over = used_bytes() + need > opt_.hbm_budget;
  const bool room = !over || make_room(need, r.pid);
  if (over) {
    const double dt = now_ms() - t_room;
    st_.worker_ms[2] += dt;
    st_.worker_max_ms[2] = std::max(st_.worker_max_ms[2], dt);
  }
  if (!room) {
    if (flights_.empty() && spills_.empty()) {
      // nothing in flight will free memory: the request cannot fit
      Completion c{r.ticket, r.pid, r.kind, ST_ENOMEM, 0, 0, r.t_submit, now_ms(), now_ms()};
      put_event(r.ready);
      set_error("request does not fit the HBM budget");
      push_completion(c);
      return true;
    }
    std::lock_guard<std::mutex> g(mu_);
    st_.deferred_admissions++;
    return false;
  }
  const double t_start = now_ms();
  Flight f{r, nullptr, t_start, 0, {}};
  p.busy = true;
  p.lru = ++tick_;
  // a failed start still completes in stream order, after what it issued
  f.start_rc = r.kind == REQ_CHECKPOINT ? start_checkpoint(f.r, p) : start_restart(f.r, p, &f.temps);
  {
    std::lock_guard<std::mutex> g(mu_);
    f.done = get_event();
  }
  cudaEventRecord(f.done, p.s);
  flights_.push_back(f);
  std::lock_guard<std::mutex> g(mu_);
  const double dt = now_ms() - t_start;
  st_.worker_ms[0] += dt;
  st_.worker_max_ms[0] = std::max(st_.worker_max_ms[0], dt);
  st_.inflight_peak = std::max<uint32_t>(st_.inflight_peak, (uint32_t)flights_.size());
  const uint64_t u = used_bytes();
  st_.hbm_used = u;
  st_.hbm_peak = std::max(st_.hbm_peak, u);
  return true;
}

void Server::finish(Flight& f) {
  Proc& p = *view_[f.r.pid];
  Engine& e = *p.eng;
  Completion c{f.r.ticket, f.r.pid, f.r.kind, ST_OK, 0, 0, f.r.t_submit, f.t_admit, 0};
  if (f.start_rc) {
    c.status = f.start_rc;
    set_error(e.last_error);
  } else if (f.r.kind == REQ_CHECKPOINT) {
    HeaderHost h{};
    int rc;
    {
      StepTimer t("complete", f.r.pid);
      rc = e.complete(f.r.len, &h);
      e.release_retired();
    }
    c.status = rc;
    if (rc == ST_OK) {
      const uint64_t n = e.diff_len();
      Archived a;
      a.len = n;
      a.hdr = h;
      StepTimer t_arch("archive", f.r.pid);
      if (cudaMallocFromPoolAsync(reinterpret_cast<void**>(&a.dev), n ? n : 1, pool_, p.s) == cudaSuccess) {
        archive_copy(a.dev, e.diff_device(), n, p.s);
      } else {
        // no device memory for the archive: keep it in pinned host memory
        cudaGetLastError();
        a.dev = nullptr;
        a.host = arena_.alloc(n);
        if (a.host) cudaMemcpyAsync(a.host, e.diff_device(), n, cudaMemcpyDeviceToHost, p.s);
        else c.status = ST_ENOMEM;
      }
      if (c.status == ST_OK) {
        c.chkpt_id = (uint32_t)p.chain.size();
        c.diff_len = n;
        std::lock_guard<std::mutex> g(mu_);
        p.chain.push_back(a);
        p.last_diff = n;
        if (a.dev) {
          chain_dev_ += n;
          p.chain_dev += n;
        }
        st_.checkpoints++;
        st_.bytes_checkpointed += f.r.len;
      }
      e.current_id += 1;  // checkpoint(data, len, diff_h, make_baseline) advances
      // get the next incremental checkpoint ready now, between requests:
      // its allocations and its graph capture then cost the next request
      // nothing (a new input pointer or baseline still re-prepares)
      // (not under memory pressure: the process may be spilled before then)
      StepTimer t_next("next-step prepare", f.r.pid);
      if (c.status == ST_OK && opt_.use_graph && e.mode() != MODE_FULL &&
          used_bytes() < opt_.hbm_budget - opt_.hbm_budget / 10 &&
          e.prepare(f.r.data, f.r.len, false, opt_.id_headroom) == ST_OK)
        ensure_graph(p, f.r.data, f.r.len);
    } else {
      set_error(e.last_error);
    }
  } else {
    StepTimer t("restart complete", f.r.pid);
    int rc = e.restart_complete();
    c.status = rc;
    c.chkpt_id = f.r.chkpt_id;
    if (rc == ST_OK) {
      std::lock_guard<std::mutex> g(mu_);
      st_.restarts++;
      st_.bytes_restarted += f.r.len;
    } else {
      set_error(e.last_error);
    }
  }
  if (p.spill && !e.spilled()) {  // the restore's pinned copy has been read
    arena_.free(p.spill, p.spill_len);
    p.spill = nullptr;
    p.spill_len = 0;
  }
  refresh_state_bytes(p);
  p.busy = false;
  c.t_done_ms = now_ms();
  put_event(f.r.ready);
  put_event(f.done);
  push_completion(c);
}

void Server::worker() {
  cudaSetDevice(device_);
  while (true) {
    {
      std::unique_lock<std::mutex> g(mu_);
      if (stop_ && inbox_.empty() && pending_.empty() && flights_.empty()) break;
      if (view_.size() != procs_.size()) {
        view_.clear();
        for (auto& pp : procs_) view_.push_back(pp.get());
      }
      while (!inbox_.empty()) {
        pending_.push_back(inbox_.front());
        inbox_.pop_front();
      }
    }
    bool progress = false;
    // 0. archived checkpoints whose copy to pinned memory has landed
    if (!spills_.empty()) {
      const size_t before = spills_.size();
      reap_spills();
      progress = spills_.size() != before;
    }
    // 1. completions
    for (size_t i = 0; i < flights_.size();) {
      cudaError_t q = cudaEventQuery(flights_[i].done);
      if (q == cudaErrorNotReady) {
        i++;
        continue;
      }
      if (q != cudaSuccess) {
        flights_[i].start_rc = ST_ECUDA;
        set_error(std::string("device error: ") + cudaGetErrorString(q));
      }
      Flight f = flights_[i];
      flights_.erase(flights_.begin() + (long)i);
      const double t_fin = now_ms();
      finish(f);
      const double dt = now_ms() - t_fin;
      st_.worker_ms[1] += dt;
      st_.worker_max_ms[1] = std::max(st_.worker_max_ms[1], dt);
      progress = true;
    }
    // 2. past 90% of the budget, make room ahead of need until 87.5% stays
    //    resident: first the restart tables that idle processes keep, then
    //    the oldest archived checkpoints of the least recently used
    //    processes, a bounded amount per pass, between admissions, so that
    //    neither a request nor the worker waits for the copies
    if (used_bytes() - spilling_bytes_ > opt_.hbm_budget - opt_.hbm_budget / 10) {
      const double t_room = now_ms();
      const uint64_t low = opt_.hbm_budget - opt_.hbm_budget / 8;
      drop_scratch(low + spilling_bytes_, UINT32_MAX);
      if (spilling_bytes_ < kSpillInFlightBytes)
        spill_chains(low, UINT32_MAX, std::min(kSpillStepBytes, kSpillInFlightBytes - spilling_bytes_));
      const double dt = now_ms() - t_room;
      st_.worker_ms[2] += dt;
      st_.worker_max_ms[2] = std::max(st_.worker_max_ms[2], dt);
    }
    // 3. admission in submission order; one request per process at a time
    std::set<uint32_t> seen;
    for (auto it = pending_.begin(); it != pending_.end() && flights_.size() < opt_.max_inflight;) {
      const uint32_t pid = it->pid;
      if (seen.count(pid) || view_[pid]->busy) {
        seen.insert(pid);
        ++it;
        continue;
      }
      seen.insert(pid);
      if (try_start(*it)) {
        it = pending_.erase(it);
        progress = true;
      } else {
        ++it;
      }
    }
    if (!progress) {
      const double t_wait = now_ms();
      std::unique_lock<std::mutex> g(mu_);
      if (inbox_.empty() && !stop_)
        cv_work_.wait_for(g, flights_.empty() && spills_.empty() ? std::chrono::microseconds(2000)
                                                                 : std::chrono::microseconds(20));
      st_.worker_ms[3] += now_ms() - t_wait;
    }
  }
}

}  // namespace mtc
