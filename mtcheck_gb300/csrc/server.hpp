// server.hpp -- a request-serving loop over many deduplicators.
//
// Clients (simulated application processes) submit checkpoint and restart
// requests at any time from any thread.  One worker thread owns the GPU work:
//   * continuous admission: a request is started as soon as its process has
//     no other request on the GPU, an in-flight slot is free and its memory
//     fits the HBM budget; requests of different processes overlap on the
//     device (one CUDA stream per process), requests of one process run in
//     submission order;
//   * each process keeps its chunk digests (Merkle tree or hash list) and
//     digest map resident in HBM, plus the chain of its incremental
//     checkpoints for restarts;
//   * when the budget is exceeded the least recently used idle processes are
//     spilled to pinned host memory: first their archived checkpoints, then
//     their digest state; a spilled process is restored on its next request;
//   * incremental checkpoints of a process replay a per-process CUDA graph,
//     captured right after the previous checkpoint completes.
// Every result is the one a lone deduplicator gives for the same sequence of
// buffers: the launch sequence per process is the same, only its scheduling
// differs.
#pragma once
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.hpp"

namespace mtc {

struct ServerOptions {
  uint64_t hbm_budget = 120ull * 1000 * 1000 * 1000;
  uint32_t max_inflight = 64;
  uint32_t id_headroom = 64;
  // Per-process CUDA graphs for incremental checkpoints.  The worker
  // captures one when a process's buffers move; during that capture a
  // device-wide synchronisation by any thread of the application fails.
  int use_graph = 0;
  // Allocate the HBM budget (and an eighth more, for what its accounting
  // leaves out) from the server's pool once at creation and keep it there,
  // and pin this much host memory for spills up front:
  // growing either later costs milliseconds per allocation.  With a pinned
  // reserve, a helper thread also keeps an eighth of it unused and pinned
  // ahead of the spills.
  int reserve_hbm = 0;
  uint64_t pinned_reserve = 0;
};

enum : int { REQ_CHECKPOINT = 0, REQ_RESTART = 1 };

struct Completion {
  uint64_t ticket;
  uint32_t pid;
  int32_t kind;
  int32_t status;
  uint32_t chkpt_id;
  uint64_t diff_len;
  double t_submit_ms, t_admit_ms, t_done_ms;
};

struct ServerStats {
  uint64_t submitted = 0, completed = 0, failed = 0, checkpoints = 0, restarts = 0;
  uint64_t bytes_checkpointed = 0, bytes_restarted = 0;
  uint64_t spilled_diffs = 0, spilled_states = 0, restored_states = 0, staged_diffs = 0;
  uint64_t spilled_bytes = 0;
  uint64_t graph_captures = 0, graph_replays = 0;
  uint64_t hbm_used = 0, hbm_peak = 0, pinned_reserved = 0;
  uint64_t pinned_sync_grows = 0;  // slabs the worker had to pin itself
  uint64_t pool_reserved_high = 0, pool_used_high = 0;  // device bytes the pool mapped / handed out, peaks
  uint64_t deferred_admissions = 0;  // admission attempts refused for memory
  uint32_t inflight_peak = 0;
  double worker_ms[4] = {0, 0, 0, 0};  // host time of the worker: starting requests,
                                       // finishing them, making room, waiting
  double worker_max_ms[3] = {0, 0, 0};  // longest single start, finish, room-making pass
};

// Pinned host memory for spills, in blocks of quarter-power-of-two classes
// (64 KiB, then p, 1.25p, 1.5p, 1.75p for each power of two p: at most a
// quarter of a block is unused), reused, freed at destruction.  Blocks are
// carved from slabs of at least 256 MiB, mapped, touched and then registered
// with CUDA.  Touching a slab's pages takes tens of milliseconds, so with
// keep_spare() a helper thread prepares the next slabs while the unused slab
// space is below the given size, and the thread that allocates pins only when
// the helper has fallen behind.  All members are thread-safe.
class PinnedArena {
 public:
  ~PinnedArena();
  uint8_t* alloc(uint64_t n);
  void free(uint8_t* p, uint64_t n);
  bool reserve(uint64_t bytes);
  void keep_spare(int device, uint64_t bytes);
  uint64_t reserved();
  uint64_t sync_grows();
  static uint64_t cls(uint64_t n);

 private:
  struct Slab {
    uint8_t* next;
    uint64_t left;
  };
  bool add_slab(uint64_t bytes);
  uint8_t* carve(uint64_t c);  // caller holds mu_
  void helper(int device);
  std::mutex mu_;
  std::condition_variable cv_;
  std::thread helper_;
  bool stop_ = false;
  uint64_t spare_target_ = 0;
  uint64_t spare_ = 0;  // unused slab bytes
  std::map<uint64_t, std::vector<uint8_t*>> free_;
  std::vector<std::pair<uint8_t*, uint64_t>> all_;  // mapped and registered slabs
  std::vector<Slab> slabs_;
  uint64_t reserved_ = 0;
  uint64_t sync_grows_ = 0;
};

class Server {
 public:
  explicit Server(const ServerOptions& o);
  ~Server();
  int add_process(int mode, int hash_kind, uint32_t chunk_size, uint32_t* pid);
  int submit_checkpoint(uint32_t pid, const uint8_t* data, uint64_t len, bool make_baseline, uint64_t* ticket);
  int submit_restart(uint32_t pid, uint32_t chkpt_id, uint8_t* out, uint64_t len, uint64_t* ticket);
  // Up to `max` completions; waits up to wait_ms for the first one.
  uint32_t poll(Completion* out, uint32_t max, double wait_ms);
  // Wait until every submitted request has completed (false on timeout).
  bool drain(double timeout_ms);
  int chain_length(uint32_t pid, uint32_t* n);
  int copy_diff(uint32_t pid, uint32_t chkpt_id, void* host, uint64_t cap, uint64_t* len);
  ServerStats stats();
  std::string error();
  static double now_ms();

 private:
  struct Archived {
    uint8_t* dev = nullptr;   // pool allocation, or null when spilled
    uint8_t* host = nullptr;  // pinned copy when spilled (or being spilled)
    uint64_t len = 0;
    HeaderHost hdr{};
    bool spilling = false;    // host copy in flight; dev stays valid until it lands
  };
  // Diffs whose copy to pinned memory is in flight on the spill stream,
  // and the event recorded after their copies.  Their device blocks are
  // freed only once the copies have run: freed earlier, the pool could hand
  // a block to another process's request, which would then wait behind the
  // whole copy.
  struct SpillBatch {
    cudaEvent_t ev;
    std::vector<std::pair<uint32_t, uint32_t>> items;  // (process, chain index)
  };
  struct Proc {
    std::unique_ptr<Engine> eng;
    cudaStream_t s = nullptr;
    std::vector<Archived> chain;
    bool busy = false;
    uint64_t lru = 0;
    uint64_t state_dev = 0;        // device bytes of the engine when resident
    uint64_t scratch_dev = 0;      // restart tables the engine keeps (dropped first under pressure)
    uint8_t* spill = nullptr;      // pinned copy of the digest state
    uint64_t spill_len = 0;
    cudaGraphExec_t exec = nullptr;
    uint64_t sig = 0;
    uint64_t chain_dev = 0;        // device bytes of archived checkpoints
    uint64_t chain_moving = 0;     // of which the host copy is in flight
    uint64_t last_diff = 0;        // size of the latest incremental checkpoint
  };
  struct Req {
    uint64_t ticket;
    uint32_t pid;
    int kind;
    const uint8_t* data;
    uint8_t* out;
    uint64_t len;
    bool make_baseline;
    uint32_t chkpt_id;
    double t_submit;
    cudaEvent_t ready;
  };
  struct Flight {
    Req r;
    cudaEvent_t done;
    double t_admit;
    int start_rc;                 // nonzero: the start failed part-way
    std::vector<uint8_t*> temps;  // staged spilled diffs of a restart
  };

  void worker();
  bool try_start(Req& r);
  int start_checkpoint(Req& r, Proc& p);
  int ensure_graph(Proc& p, const uint8_t* data, uint64_t len);
  int start_restart(Req& r, Proc& p, std::vector<uint8_t*>* temps);
  void finish(Flight& f);
  uint64_t need_bytes(const Req& r, const Proc& p) const;
  bool make_room(uint64_t need, uint32_t except);
  uint64_t used_bytes() const;
  uint64_t drop_scratch(uint64_t target, uint32_t except);
  uint64_t spill_chains(uint64_t target, uint32_t except, uint64_t max_bytes);
  void reap_spills();
  void spill_state(Proc& p);
  int restore_state(Proc& p);
  void refresh_state_bytes(Proc& p);
  cudaEvent_t get_event();
  void put_event(cudaEvent_t e);
  void push_completion(const Completion& c);
  void set_error(const std::string& e);

  ServerOptions opt_;
  int device_ = 0;
  cudaMemPool_t pool_ = nullptr;
  PinnedArena arena_;
  std::vector<std::unique_ptr<Proc>> procs_;  // owned; grows under mu_
  std::vector<Proc*> view_;                   // the worker's copy of procs_
  std::deque<Req> inbox_, pending_;
  std::vector<Flight> flights_;
  std::vector<SpillBatch> spills_;  // worker thread only
  cudaStream_t spill_s_ = nullptr;  // copies of spilled diffs to pinned memory
  uint64_t spilling_bytes_ = 0;    // device bytes whose host copy is in flight
  std::deque<Completion> done_;
  std::vector<cudaEvent_t> events_;
  std::mutex mu_;                  // inbox, completions, events, procs vector, chains
  std::condition_variable cv_work_, cv_done_;
  std::thread thread_;
  std::atomic<bool> stop_{false};
  uint64_t next_ticket_ = 1, outstanding_ = 0, tick_ = 0, chain_dev_ = 0;
  ServerStats st_;
  std::string err_;
};

}  // namespace mtc
