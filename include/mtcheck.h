/*
 * mtcheck.h -- C ABI of the GB300 incremental-checkpoint deduplicator.
 *
 * Drop-in boundary for the deduplication path of TauferLab/MTCheck: each
 * entry point replaces one member of BaseDeduplicator
 * (include/deduplicator_interface.hpp:14-184) or one helper of the
 * reference, cited beside it.  Plain pointers and sizes only; "device"
 * pointers are CUDA device addresses on the current device.  Every call
 * returns an MTC_* status; mtc_last_error() gives a message for the calling
 * thread.  A handle is not thread-safe; distinct handles are independent.
 */
#ifndef MTCHECK_H
#define MTCHECK_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference reports errors only by printf) */
#define MTC_OK 0
#define MTC_EINVAL 1     /* bad argument, length change without baseline, short buffer */
#define MTC_ECORRUPT 2   /* malformed incremental checkpoint */
#define MTC_ENOMEM 3     /* device or host allocation failed, table full */
#define MTC_ETIMEOUT 4   /* a bounded device wait expired */
#define MTC_ECUDA 5      /* CUDA runtime error */
#define MTC_EINTERNAL 6  /* internal invariant violated */
#define MTC_ENOTSUP 7    /* outside the supported range */

/* approaches: DedupMode values of include/utils.hpp:39-49 */
#define MTC_FULL 1
#define MTC_BASIC 2
#define MTC_LIST 3
#define MTC_TREE 4
#define MTC_TREE_LOW_OFFSET_REF 5 /* tree with the serial labelling of include/reference_impl.hpp:16-132 */
#define MTC_TREE_LOW_OFFSET 6     /* same as MTC_TREE (src/dedup_files.cpp:68-70) */

/* chunk digest functions: include/hash_functions.hpp:16-20 selects one at build time */
#define MTC_HASH_MURMUR3 0 /* include/kokkos_murmur3.hpp:213-292, 431-437 */
#define MTC_HASH_MD5 1     /* include/kokkos_md5.hpp:287-323 */

/* header_t, include/utils.hpp:29-37: the first 32 bytes of every .basic,
 * .hashlist and .hashtree incremental checkpoint */
typedef struct mtc_header {
  uint32_t ref_id;
  uint32_t chkpt_id;
  uint64_t datalen;
  uint32_t chunk_size;
  uint32_t num_first_ocur;
  uint32_t num_prior_chkpts;
  uint32_t num_shift_dupl;
} mtc_header_t;

/* counters and timers of the last operation (BaseDeduplicator members
 * current_id, baseline_id, datasizes, timers[4], restart_timers[2],
 * include/deduplicator_interface.hpp:15-23; TreeDeduplicator::num_first_ocur /
 * num_shift_dupl, include/tree_approach.hpp:52-58) */
typedef struct mtc_info {
  uint32_t current_id;
  uint32_t baseline_id;
  uint32_t chunk_size;
  uint32_t num_first_ocur;
  uint32_t num_shift_dupl;
  uint32_t num_prior_chkpts;
  uint64_t data_len;
  uint64_t diff_len;
  uint64_t data_size;      /* datasizes.first */
  uint64_t metadata_size;  /* datasizes.second */
  double timers[4];        /* setup, compare, gather, copy to host (s) */
  double restart_timers[2];/* copy, total (s) */
  double phase_times[3];   /* device time of the last checkpoint: leaf hashing kernel,
                              forest passes and root compaction, diff assembly (s) */
  uint32_t device_error;   /* last device error bits (0 = none) */
  uint32_t reserved;
} mtc_info_t;

typedef struct mtc_dedup mtc_dedup_t;

/* TreeDeduplicator(uint32_t) and siblings, src/tree_approach.cpp:5-9 */
int mtc_create(int approach, int hash, uint32_t chunk_size, mtc_dedup_t** out);
/* ~TreeDeduplicator(), src/tree_approach.cpp:11 */
int mtc_destroy(mtc_dedup_t* h);
/* CUDA stream for all work of the handle (0 = legacy default stream); the
 * reference uses Kokkos' default execution space instance */
int mtc_set_stream(mtc_dedup_t* h, void* cuda_stream);

/* checkpoint(header_t&, uint8_t*, size_t, HostMirror&, bool),
 * include/deduplicator_interface.hpp:52-57: deduplicates the device buffer and
 * assembles the incremental checkpoint in device memory; current_id is NOT
 * advanced.  *diff_len receives its size; fetch it with mtc_diff_copy. */
int mtc_checkpoint_header(mtc_dedup_t* h, mtc_header_t* header, const void* dev_data, uint64_t len,
                          int make_baseline, uint64_t* diff_len);
/* checkpoint(uint8_t*, size_t, HostMirror&, bool), :93-96 (advances current_id) */
int mtc_checkpoint(mtc_dedup_t* h, const void* dev_data, uint64_t len, int make_baseline, uint64_t* diff_len);
/* Fault injection for failure-detection tests (no reference counterpart):
 * the next `checkpoints` checkpoints of the handle run with the copy producer
 * of the chunk-hashing kernel silent, so the kernel's bounded waits run out
 * (after about a millisecond) and the call returns MTC_ETIMEOUT; the GPU
 * context stays usable.  After any MTC_ETIMEOUT from a checkpoint the
 * handle's digest state may be partly updated, so its next checkpoint is
 * taken as a baseline (as if make_baseline were set). */
int mtc_inject_stall(mtc_dedup_t* h, uint32_t checkpoints);
/* current_id += 1: what the reference's convenience overloads do after
 * checkpoint(header_t&, ...) (src/tree_approach.cpp:1723, :1747, :1775) */
int mtc_advance(mtc_dedup_t* h);
/* the device->host copy of the diff, src/tree_approach.cpp:1677-1688 */
int mtc_diff_copy(mtc_dedup_t* h, void* host_dst, uint64_t capacity);
/* the diff of the last checkpoint in device memory (valid until the next call) */
int mtc_diff_device(mtc_dedup_t* h, const void** dev_ptr, uint64_t* len);
/* checkpoint + malloc'd host copy (release with mtc_free); advances current_id */
int mtc_checkpoint_alloc(mtc_dedup_t* h, const void* dev_data, uint64_t len, int make_baseline, void** host_diff,
                         uint64_t* diff_len);
void mtc_free(void* p);
/* checkpoint(uint8_t*, size_t, std::string& filename, std::string& logname, bool),
 * :73-77: writes the diff to `filename` and the CSV logs under `logname`
 * (logname NULL: no logs) */
int mtc_checkpoint_file(mtc_dedup_t* h, const void* dev_data, uint64_t len, const char* filename,
                        const char* logname, int make_baseline);

/* restart(uint8_t*, size_t, std::vector<HostMirror>&, std::string&, uint32_t),
 * :142-146: rebuilds checkpoint `chkpt_id` of the chain `host_diffs[0..n)` into
 * the device buffer `dev_out` of `len` == header.datalen bytes.  Where the GPU
 * can read the host memory (pinned memory; pageable memory on a system with
 * cudaDevAttrPageableMemoryAccess, such as Grace), the kernels read the chain
 * in place; elsewhere, or with MTCHECK_RESTART_HOST=stage in the environment,
 * the chain is first copied to device memory.  Returns when the restart is
 * complete; the host buffers may be released then. */
int mtc_restart(mtc_dedup_t* h, void* dev_out, uint64_t len, const void* const* host_diffs, const uint64_t* lens,
                uint32_t n, uint32_t chkpt_id);
/* same, with the chain already resident in device memory; the diffs must be
 * complete in the order of the handle's stream (their headers are read on it) */
int mtc_restart_device(mtc_dedup_t* h, void* dev_out, uint64_t len, const void* const* dev_diffs,
                       const uint64_t* lens, uint32_t n, uint32_t chkpt_id);
/* restart(View, std::vector<std::string>& filenames, std::string&, uint32_t), :156-159;
 * the names are complete paths of the incremental checkpoint files */
int mtc_restart_files(mtc_dedup_t* h, void* dev_out, uint64_t len, const char* const* filenames, uint32_t n,
                      uint32_t chkpt_id);
/* A handle keeps its restart tables between restarts (about 16 bytes per
 * chunk per chain step, plus about 100 bytes per chunk); this frees them.
 * The next restart allocates them again.  No reference counterpart. */
int mtc_release_restart_buffers(mtc_dedup_t* h);

/* counters and timers */
int mtc_get_info(const mtc_dedup_t* h, mtc_info_t* out);
/* write_chkpt_log(header_t&, HostMirror& diff_h, std::string& logname),
 * include/deduplicator_interface.hpp:172-174: appends the three CSV logs
 * <logname>.chunk_size.<c>{.csv,.size.csv,.timing.csv} for the last checkpoint */
int mtc_write_chkpt_log(const mtc_dedup_t* h, const mtc_header_t* header, const void* host_diff, uint64_t len,
                        const char* logname);
/* write_restart_log(uint32_t select_chkpt, std::string& logname), :181-183 */
int mtc_write_restart_log(const mtc_dedup_t* h, uint32_t select_chkpt, const char* logname);

/* chunk digests of a device buffer into dev_digests (16 bytes per chunk, the
 * last chunk may be short): the per-chunk hash() calls of the leaf loops,
 * src/tree_approach.cpp:319-323 */
int mtc_hash_chunks(int hash, const void* dev_data, uint64_t len, uint32_t chunk_size, void* dev_digests,
                    void* cuda_stream);
/* calculate_digest_host's digest, include/hash_functions.hpp:65-82 */
int mtc_digest_host(int hash, const void* host_data, uint64_t len, uint8_t out[16]);
/* its printable form: "XXXXXXXX XXXXXXXX XXXXXXXX XXXXXXXX " (37 bytes incl. NUL) */
int mtc_digest_hex(const uint8_t digest[16], char out[37]);

/* Checkpoint for callers that cannot allocate memory.  No counterpart in
 * the reference.  It serves code that must not or cannot allocate: an
 * out-of-memory handler saving state when no memory is left to ask for, a
 * signal or crash handler taking a last checkpoint without entering an
 * allocator that may be locked or corrupt, and a runtime or custom allocator
 * whose pool owns the whole GPU (a cudaMalloc there would recurse into it).
 * It produces the same bytes as the basic approach (MTC_BASIC) without a
 * handle, calls no cudaMalloc, cudaFree or other allocating routine, and
 * takes no host heap memory of its own:
 *   dev_digests  caller-owned, 16-byte aligned, 16 bytes per chunk; the
 *                previous checkpoint's chunk digests on entry (any value
 *                before the first), the current ones on return
 *   first        nonzero for the first checkpoint (every chunk is saved)
 *   dev_diff     caller-owned device buffer, 4-byte aligned, capacity at least
 *                32 + chunks * (4 + chunk_size); receives the .basic checkpoint
 *                (header with ref_id/chkpt_id as given, changed chunk ids in
 *                ascending order, their data)
 * At most 4194304 chunks per call (MTC_ENOTSUP beyond).  Its scratch is a
 * fixed device array of about 4 MiB in the library, which every GPU that
 * loads the library holds until the process exits.  The first call on each
 * device does the set-up: it looks up that array's device address (and the
 * CUDA driver loads the kernels it uses), so make that first call early, while
 * memory is still available, and before any stream capture.  The call
 * synchronises its stream (it reads the count of changed chunks back), so it
 * must not be made while a capture is active on that stream.  Calls share
 * the array and each keeps the last call's contents: calls that overlap on
 * the GPU (other streams or threads) race and must be serialised by the
 * caller.  A bounded device wait that runs out gives MTC_ETIMEOUT. */
int mtc_basic_checkpoint_noalloc(int hash, const void* dev_data, uint64_t len, uint32_t chunk_size,
                                 void* dev_digests, uint32_t ref_id, uint32_t chkpt_id, int first, void* dev_diff,
                                 uint64_t diff_capacity, uint64_t* diff_len, void* cuda_stream);

/* ---- batched checkpoints (no counterpart in the reference: its drivers
 * checkpoint one buffer per call, src/dedup_files.cpp:86-102) ----
 * A batch holds n deduplicators of any approach, hash and chunk size, each on
 * its own stream.  mtc_batch_checkpoint checkpoints every member in one call:
 * the baseline step runs eagerly with all members overlapped; later steps
 * replay one CUDA graph holding every member's kernels as parallel branches
 * (captured again only when a member's device buffers move).  Each member's
 * diff, header and counters are byte-identical to those of a lone handle
 * given the same buffers; read them through the member handles. */
typedef struct mtc_batch mtc_batch_t;
typedef struct mtc_batch_info {
  uint64_t steps;
  uint64_t graph_captures;
  uint64_t graph_nodes;
  uint64_t kernels_per_step;
  double last_device_ms;   /* fork to join of the last step (CUDA events) */
  double last_call_ms;     /* host wall time of the last mtc_batch_checkpoint */
  double host_ms[5];       /* its parts: prepare (allocation, validation), graph
                              capture, issue, wait for the join, completion */
  int32_t last_used_graph;
  uint32_t batched_leaf_members; /* members whose leaves ran in the one persistent
                                    launch of the last graph step (its work queue
                                    holds their (member, tile) items) */
} mtc_batch_info_t;
int mtc_batch_create(uint32_t n, const int* approaches, const int* hashes, const uint32_t* chunk_sizes,
                     mtc_batch_t** out);
int mtc_batch_destroy(mtc_batch_t* b);
/* member i as an ordinary handle (owned by the batch: do not mtc_destroy it;
 * mtc_set_stream on it is refused) */
int mtc_batch_member(mtc_batch_t* b, uint32_t i, mtc_dedup_t** member);
/* checkpoint(data_i, len_i, diff_h, make_baseline) of every member, current_id
 * advanced; diff_lens (may be NULL) receives the n diff sizes */
int mtc_batch_checkpoint(mtc_batch_t* b, const void* const* dev_data, const uint64_t* lens, int make_baseline,
                         uint64_t* diff_lens);
/* use_graph 0: issue every step eagerly (still overlapped across members);
 * id_headroom: checkpoint ids one captured graph serves before re-capture */
int mtc_batch_set_options(mtc_batch_t* b, int use_graph, uint32_t id_headroom);
int mtc_batch_get_info(const mtc_batch_t* b, mtc_batch_info_t* out);
/* run the autotuner for every member (cached per approach, hash, chunk size
 * and power-of-two length; lengths above 64 MiB share one 64 MiB trial) and
 * apply the winners */
int mtc_batch_autotune(mtc_batch_t* b, const uint64_t* lens);
/* reserve device memory, now, for every member's state on buffers of these
 * lengths (the members' pool keeps it), so that the first checkpoint does not
 * grow the pool; *bytes (may be NULL) receives the amount reserved */
int mtc_batch_reserve(mtc_batch_t* b, const uint64_t* lens, uint64_t* bytes);

/* ---- request serving (no counterpart in the reference: its MPI driver runs
 * one process per rank, src/dedup_files_mpi.cpp:54-120) ----
 * A server owns many deduplicators ("processes") and one worker thread that
 * admits checkpoint and restart requests continuously: a request starts when
 * its process has nothing else on the GPU, an in-flight slot is free and its
 * memory fits the HBM budget, so requests of different processes overlap on
 * the device.  Each process keeps its digest state and its chain of
 * incremental checkpoints in HBM; beyond the budget the least recently used
 * idle processes spill (archived checkpoints first, then digest state) to
 * pinned host memory and come back on their next request.  Results equal
 * those of a lone handle given the same requests in the same order.
 * Inputs are read after the work already issued to the legacy default stream
 * when the request was submitted; they must not change until it completes. */
typedef struct mtc_server mtc_server_t;
typedef struct mtc_server_options {
  uint64_t hbm_budget;     /* bytes of device memory for all process state (0: 120 GB) */
  uint32_t max_inflight;   /* requests on the GPU at once (0: 64) */
  uint32_t id_headroom;    /* checkpoint ids one captured graph serves (0: 64) */
  int32_t use_graph;       /* replay a per-process CUDA graph for incremental checkpoints;
                              while the worker captures one, no thread of the application
                              may synchronise the whole device (cudaDeviceSynchronize) */
  int32_t reserve_hbm;     /* take the whole budget from the device at creation */
  uint64_t pinned_reserve; /* bytes of pinned host memory for spills, pinned at creation;
                              a helper thread then keeps an eighth of it pinned ahead of use */
} mtc_server_options_t;
#define MTC_REQ_CHECKPOINT 0
#define MTC_REQ_RESTART 1
typedef struct mtc_completion {
  uint64_t ticket;
  uint32_t pid;
  int32_t kind;            /* MTC_REQ_* */
  int32_t status;          /* MTC_* */
  uint32_t chkpt_id;       /* checkpoint written, or restarted */
  uint64_t diff_len;       /* size of the incremental checkpoint written */
  double t_submit_ms, t_admit_ms, t_done_ms;  /* mtc_now_ms() clock */
} mtc_completion_t;
typedef struct mtc_server_stats {
  uint64_t submitted, completed, failed, checkpoints, restarts;
  uint64_t bytes_checkpointed, bytes_restarted;
  uint64_t spilled_diffs, spilled_states, restored_states, staged_diffs, spilled_bytes;
  uint64_t graph_captures, graph_replays;
  uint64_t hbm_used, hbm_peak, pinned_reserved, deferred_admissions;
  uint64_t pool_reserved_high, pool_used_high; /* device bytes the server's pool mapped and
                                                  handed out, highest so far */
  uint32_t inflight_peak;
  uint32_t pinned_sync_grows; /* pinned slabs the worker thread had to pin itself */
  double worker_ms[4];     /* worker host time: starting requests, finishing them,
                              making room (spills), waiting for work */
  double worker_max_ms[3]; /* longest single start, finish and room-making pass */
} mtc_server_stats_t;
int mtc_server_create(const mtc_server_options_t* opt, mtc_server_t** out);
/* waits for every submitted request, then frees everything */
int mtc_server_destroy(mtc_server_t* s);
int mtc_server_add_process(mtc_server_t* s, int approach, int hash, uint32_t chunk_size, uint32_t* pid);
/* checkpoint(data, len, diff_h, make_baseline) of process pid; the
 * incremental checkpoint is kept in the process's chain */
int mtc_server_submit_checkpoint(mtc_server_t* s, uint32_t pid, const void* dev_data, uint64_t len,
                                 int make_baseline, uint64_t* ticket);
/* restart of checkpoint chkpt_id of process pid into dev_out (len bytes) */
int mtc_server_submit_restart(mtc_server_t* s, uint32_t pid, uint32_t chkpt_id, void* dev_out, uint64_t len,
                              uint64_t* ticket);
/* up to max completions into out (*n of them), waiting up to wait_ms for one */
int mtc_server_poll(mtc_server_t* s, mtc_completion_t* out, uint32_t max, uint32_t* n, double wait_ms);
/* wait until every submitted request has completed (MTC_ETIMEOUT on timeout) */
int mtc_server_drain(mtc_server_t* s, double timeout_ms);
int mtc_server_chain_length(mtc_server_t* s, uint32_t pid, uint32_t* n);
/* copy checkpoint chkpt_id of process pid to host memory (host NULL: size only) */
int mtc_server_copy_diff(mtc_server_t* s, uint32_t pid, uint32_t chkpt_id, void* host, uint64_t capacity,
                         uint64_t* len);
int mtc_server_get_stats(mtc_server_t* s, mtc_server_stats_t* out);
/* the clock of the completion times (milliseconds, monotonic) */
double mtc_now_ms(void);

/* ---- launch tuning (no counterpart in the reference) ----
 * Shape of the chunk-hashing kernel and the digest map's load factor.  Any
 * setting gives identical output; only the speed changes. */
typedef struct mtc_tune {
  int32_t rows;         /* chunks per CTA tile: 128 or 256 */
  int32_t ctas_per_sm;  /* 0: as many as fit (at most 3) */
  int32_t direct;       /* 1: per-thread global loads instead of TMA staging */
  int32_t eager;        /* 1: issue every launch of a checkpoint from the host instead of
                           replaying the captured sequence (single-handle calls) */
  double max_load;      /* digest-map load factor bound, (0.1, 0.95] */
  int32_t threads_per_chunk; /* 1 (0 taken as 1): one thread per chunk; 32: one warp
                                per chunk (chunks of at most 4096 bytes; the warp loads
                                the chunk, one lane hashes it: the digests are serial) */
  int32_t untimed;      /* 1: replay an incremental checkpoint as one graph, without the
                           events between its phases (one graph launch instead of five);
                           the phase times and the log timers then read 0 */
} mtc_tune_t;
int mtc_set_tuning(mtc_dedup_t* h, const mtc_tune_t* t);
int mtc_get_tuning(const mtc_dedup_t* h, mtc_tune_t* out);
/* time the candidate shapes on a seeded synthetic buffer of `len` bytes
 * (allocated and freed inside) and return the fastest; best_ms and
 * default_ms (may be NULL) receive the mean incremental checkpoint device
 * time of the winner and of the default shape */
int mtc_autotune(int approach, int hash, uint32_t chunk_size, uint64_t len, mtc_tune_t* best, double* best_ms,
                 double* default_ms);

/* kernels launched by the library so far (all handles) */
uint64_t mtc_launch_count(void);
/* message for the last failing call on this thread */
const char* mtc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* MTCHECK_H */
