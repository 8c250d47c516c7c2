// capi.cu -- the extern "C" boundary declared in include/mtcheck.h.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/mtcheck.h"
#include "batch.hpp"
#include "engine.hpp"
#include "server.hpp"
#include "host_digest.hpp"
#include "logs.hpp"

struct mtc_dedup {
  mtc::Engine* eng;
  bool borrowed = false;  // a batch member: the batch owns the engine
};

struct mtc_server {
  mtc::Server* s = nullptr;
};

struct mtc_batch {
  mtc::Batch* b = nullptr;
  std::vector<mtc_dedup> members;
};

namespace {
// The message of the last failing call on this thread, in a fixed array (no
// heap allocation when a call fails).
constexpr size_t kErrCap = 512;
thread_local char t_err[kErrCap];

int ret(int rc, const char* msg) {
  if (rc != MTC_OK) mtc::set_last_error(msg);
  return rc;
}
int ret(int rc, const std::string& msg) { return ret(rc, msg.c_str()); }
int ret_eng(int rc, mtc::Engine* e) { return ret(rc, e ? e->last_error.c_str() : "error"); }

bool valid_mode(int a) { return a >= MTC_FULL && a <= MTC_TREE_LOW_OFFSET; }
}  // namespace

void mtc::set_last_error(const char* msg) {
  if (!msg) msg = "";
  size_t n = std::strlen(msg);
  if (n >= kErrCap) n = kErrCap - 1;
  std::memcpy(t_err, msg, n);
  t_err[n] = 0;
}

extern "C" {

int mtc_create(int approach, int hash, uint32_t chunk_size, mtc_dedup_t** out) {
  if (!out) return ret(MTC_EINVAL, "out is NULL");
  *out = nullptr;
  if (!valid_mode(approach)) return ret(MTC_EINVAL, "unknown approach");
  if (hash != MTC_HASH_MURMUR3 && hash != MTC_HASH_MD5) return ret(MTC_EINVAL, "unknown hash");
  if (chunk_size == 0) return ret(MTC_EINVAL, "chunk size is 0");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ret(MTC_ECUDA, "no CUDA device");
  auto* h = new (std::nothrow) mtc_dedup;
  if (!h) return ret(MTC_ENOMEM, "out of host memory");
  h->eng = new (std::nothrow) mtc::Engine(approach, hash, chunk_size);
  if (!h->eng) { delete h; return ret(MTC_ENOMEM, "out of host memory"); }
  *out = h;
  return MTC_OK;
}

int mtc_destroy(mtc_dedup_t* h) {
  if (!h) return MTC_OK;
  if (h->borrowed) return ret(MTC_EINVAL, "batch members are destroyed with their batch");
  delete h->eng;
  delete h;
  return MTC_OK;
}

int mtc_set_stream(mtc_dedup_t* h, void* s) {
  if (!h) return ret(MTC_EINVAL, "NULL handle");
  if (h->borrowed) return ret(MTC_EINVAL, "a batch member runs on the batch's stream");
  h->eng->set_stream(reinterpret_cast<cudaStream_t>(s));
  return MTC_OK;
}

int mtc_checkpoint_header(mtc_dedup_t* h, mtc_header_t* header, const void* dev_data, uint64_t len,
                          int make_baseline, uint64_t* diff_len) {
  if (!h) return ret(MTC_EINVAL, "NULL handle");
  mtc::HeaderHost hh{};
  int rc = h->eng->checkpoint(static_cast<const uint8_t*>(dev_data), len, make_baseline != 0, &hh);
  if (rc) return ret_eng(rc, h->eng);
  if (header) std::memcpy(header, &hh, sizeof(hh));
  if (diff_len) *diff_len = h->eng->diff_len();
  return MTC_OK;
}

int mtc_checkpoint(mtc_dedup_t* h, const void* dev_data, uint64_t len, int make_baseline, uint64_t* diff_len) {
  int rc = mtc_checkpoint_header(h, nullptr, dev_data, len, make_baseline, diff_len);
  if (rc == MTC_OK) h->eng->current_id += 1;
  return rc;
}

int mtc_inject_stall(mtc_dedup_t* h, uint32_t checkpoints) {
  if (!h) return ret(MTC_EINVAL, "NULL handle");
  h->eng->inject_stall(checkpoints);
  return MTC_OK;
}

int mtc_advance(mtc_dedup_t* h) {
  if (!h) return ret(MTC_EINVAL, "NULL handle");
  h->eng->current_id += 1;
  return MTC_OK;
}

int mtc_diff_copy(mtc_dedup_t* h, void* host_dst, uint64_t capacity) {
  if (!h || !host_dst) return ret(MTC_EINVAL, "NULL argument");
  return ret_eng(h->eng->copy_diff(host_dst, capacity), h->eng);
}

int mtc_diff_device(mtc_dedup_t* h, const void** dev_ptr, uint64_t* len) {
  if (!h || !dev_ptr || !len) return ret(MTC_EINVAL, "NULL argument");
  *dev_ptr = h->eng->diff_device();
  *len = h->eng->diff_len();
  return *dev_ptr ? MTC_OK : ret(MTC_EINVAL, "no checkpoint staged");
}

int mtc_checkpoint_alloc(mtc_dedup_t* h, const void* dev_data, uint64_t len, int make_baseline, void** host_diff,
                         uint64_t* diff_len) {
  if (!h || !host_diff) return ret(MTC_EINVAL, "NULL argument");
  *host_diff = nullptr;
  uint64_t n = 0;
  int rc = mtc_checkpoint_header(h, nullptr, dev_data, len, make_baseline, &n);
  if (rc) return rc;
  void* buf = std::malloc(n ? n : 1);
  if (!buf) return ret(MTC_ENOMEM, "out of host memory");
  rc = h->eng->copy_diff(buf, n);
  if (rc) { std::free(buf); return ret_eng(rc, h->eng); }
  h->eng->current_id += 1;
  *host_diff = buf;
  if (diff_len) *diff_len = n;
  return MTC_OK;
}

void mtc_free(void* p) { std::free(p); }

int mtc_checkpoint_file(mtc_dedup_t* h, const void* dev_data, uint64_t len, const char* filename,
                        const char* logname, int make_baseline) {
  if (!h || !filename) return ret(MTC_EINVAL, "NULL argument");
  mtc::HeaderHost hh{};
  int rc = h->eng->checkpoint(static_cast<const uint8_t*>(dev_data), len, make_baseline != 0, &hh);
  if (rc) return ret_eng(rc, h->eng);
  std::vector<uint8_t> buf(h->eng->diff_len());
  rc = h->eng->copy_diff(buf.data(), buf.size());
  if (rc) return ret_eng(rc, h->eng);
  if (logname) mtc::write_chkpt_log(*h->eng, hh, buf.data(), buf.size(), logname);
  std::ofstream f(filename, std::ios::out | std::ios::binary | std::ios::trunc);
  if (!f) return ret(MTC_EINVAL, std::string("cannot open ") + filename);
  f.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)buf.size());
  f.flush();
  if (!f) return ret(MTC_EINVAL, std::string("cannot write ") + filename);
  h->eng->current_id += 1;  // src/tree_approach.cpp:1723
  return MTC_OK;
}

int mtc_restart_device(mtc_dedup_t* h, void* dev_out, uint64_t len, const void* const* dev_diffs,
                       const uint64_t* lens, uint32_t n, uint32_t chkpt_id) {
  if (!h || !dev_out || !dev_diffs || !lens) return ret(MTC_EINVAL, "NULL argument");
  if (chkpt_id >= n) return ret(MTC_EINVAL, "checkpoint id outside the chain");
  std::vector<const uint8_t*> ptrs(n);
  std::vector<uint64_t> l(lens, lens + n);
  std::vector<mtc::HeaderHost> hdrs(n);
  for (uint32_t i = 0; i < n; i++) ptrs[i] = static_cast<const uint8_t*>(dev_diffs[i]);
  // the headers of the whole chain in one gather and one copy (a 32-byte
  // copy per diff cost about 10 us each)
  if (h->eng->mode() != MTC_FULL) {
    const int rc = h->eng->read_headers(ptrs, l, hdrs);
    if (rc) return ret_eng(rc, h->eng);
  }
  return ret_eng(h->eng->restart(static_cast<uint8_t*>(dev_out), len, ptrs, l, hdrs, chkpt_id), h->eng);
}

int mtc_release_restart_buffers(mtc_dedup_t* h) {
  if (!h) return ret(MTC_EINVAL, "NULL argument");
  h->eng->release_restart_scratch();
  return MTC_OK;
}

namespace {
// Can the restart kernels read this host memory in place?  Pinned memory
// always can (through its device alias); ordinary pageable memory can on a
// system whose GPU reads the host's page tables (NVLink-C2C with ATS on
// Grace, cudaDevAttrPageableMemoryAccess).
const uint8_t* device_view(const void* host) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, host) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
    return static_cast<const uint8_t*>(at.devicePointer);
  cudaGetLastError();
  static int pageable = -1;
  if (pageable < 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) v = 0;
    pageable = v;
  }
  return pageable ? static_cast<const uint8_t*>(host) : nullptr;
}
bool restart_in_place() {
  const char* e = std::getenv("MTCHECK_RESTART_HOST");
  return !(e && std::strcmp(e, "stage") == 0);
}
}  // namespace

int mtc_restart(mtc_dedup_t* h, void* dev_out, uint64_t len, const void* const* host_diffs, const uint64_t* lens,
                uint32_t n, uint32_t chkpt_id) {
  if (!h || !dev_out || !host_diffs || !lens) return ret(MTC_EINVAL, "NULL argument");
  if (chkpt_id >= n) return ret(MTC_EINVAL, "checkpoint id outside the chain");
  std::vector<mtc::HeaderHost> hdrs(n);
  std::vector<const uint8_t*> ptrs(n, nullptr);
  std::vector<uint64_t> l(lens, lens + n);
  uint64_t total = 0;
  for (uint32_t i = 0; i < n; i++) {
    if (h->eng->mode() != MTC_FULL && l[i] >= sizeof(mtc::HeaderHost)) std::memcpy(&hdrs[i], host_diffs[i], sizeof(mtc::HeaderHost));
    else std::memset(&hdrs[i], 0, sizeof(hdrs[i]));
    if (i <= chkpt_id) total += (l[i] + 255) & ~uint64_t(255);
  }
  // In place: the kernels read the chain where it lies in host memory, only
  // the bytes the restart needs (the metadata and each restored chunk once)
  // instead of a copy of the whole used chain; where the GPU cannot read the
  // host memory, the chain is staged in device memory first.  The reference
  // copies each diff to the device as it walks the chain
  // (src/tree_approach.cpp:756, :962).
  bool direct = restart_in_place() && h->eng->mode() != MTC_FULL;
  for (uint32_t i = 0; direct && i <= chkpt_id; i++) {
    ptrs[i] = device_view(host_diffs[i]);
    if (!ptrs[i] && l[i]) direct = false;
  }
  if (direct) {
    int rc = h->eng->restart(static_cast<uint8_t*>(dev_out), len, ptrs, l, hdrs, chkpt_id);
    if (rc == MTC_OK) h->eng->restart_timers[0] = 0;  // no staging copy
    return ret_eng(rc, h->eng);
  }
  // a staging buffer kept by the handle: no allocation, and no cudaFree
  // (which would wait for the whole device), per call
  cudaStream_t s = h->eng->stream();
  if (h->eng->restart_stage.ensure(total ? total : 1, s) != cudaSuccess) {
    cudaGetLastError();
    return ret(MTC_ENOMEM, "cannot stage the chain");
  }
  uint8_t* dev = h->eng->restart_stage.p;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, s);
  uint64_t off = 0;
  for (uint32_t i = 0; i <= chkpt_id; i++) {
    ptrs[i] = dev + off;
    if (l[i]) cudaMemcpyAsync(dev + off, host_diffs[i], l[i], cudaMemcpyHostToDevice, s);
    off += (l[i] + 255) & ~uint64_t(255);
  }
  cudaEventRecord(b, s);
  int rc = h->eng->restart(static_cast<uint8_t*>(dev_out), len, ptrs, l, hdrs, chkpt_id);
  float ms = 0;
  cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b);
  if (rc == MTC_OK) {
    h->eng->restart_timers[0] = ms * 1e-3;
    h->eng->restart_timers[1] += ms * 1e-3;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ret_eng(rc, h->eng);
}

int mtc_restart_files(mtc_dedup_t* h, void* dev_out, uint64_t len, const char* const* filenames, uint32_t n,
                      uint32_t chkpt_id) {
  if (!h || !filenames) return ret(MTC_EINVAL, "NULL argument");
  std::vector<std::vector<uint8_t>> bufs(n);
  std::vector<const void*> ptrs(n);
  std::vector<uint64_t> lens(n);
  for (uint32_t i = 0; i < n; i++) {
    std::ifstream f(filenames[i], std::ios::in | std::ios::binary | std::ios::ate);
    if (!f) return ret(MTC_EINVAL, std::string("cannot open ") + filenames[i]);
    std::streamsize sz = f.tellg();
    f.seekg(0);
    bufs[i].resize((size_t)sz);
    if (sz && !f.read(reinterpret_cast<char*>(bufs[i].data()), sz)) return ret(MTC_EINVAL, std::string("cannot read ") + filenames[i]);
    ptrs[i] = bufs[i].data();
    lens[i] = (uint64_t)sz;
  }
  return mtc_restart(h, dev_out, len, ptrs.data(), lens.data(), n, chkpt_id);
}

int mtc_get_info(const mtc_dedup_t* h, mtc_info_t* o) {
  if (!h || !o) return ret(MTC_EINVAL, "NULL argument");
  const mtc::Engine& e = *h->eng;
  std::memset(o, 0, sizeof(*o));
  o->current_id = e.current_id;
  o->baseline_id = e.baseline_id;
  o->chunk_size = e.chunk_size();
  o->num_first_ocur = e.num_first_ocur;
  o->num_shift_dupl = e.num_shift_dupl;
  o->num_prior_chkpts = e.num_prior_chkpts;
  o->data_len = e.data_len;
  o->diff_len = e.diff_len();
  o->data_size = e.datasizes[0];
  o->metadata_size = e.datasizes[1];
  for (int i = 0; i < 4; i++) o->timers[i] = e.timers[i];
  o->restart_timers[0] = e.restart_timers[0];
  o->restart_timers[1] = e.restart_timers[1];
  for (int i = 0; i < 3; i++) o->phase_times[i] = e.phase_times[i];
  o->device_error = e.last_device_error;
  return MTC_OK;
}

int mtc_write_chkpt_log(const mtc_dedup_t* h, const mtc_header_t* header, const void* host_diff, uint64_t len,
                        const char* logname) {
  if (!h || !header || !logname || (!host_diff && len)) return ret(MTC_EINVAL, "NULL argument");
  mtc::HeaderHost hh;
  std::memcpy(&hh, header, sizeof(hh));
  mtc::write_chkpt_log(*h->eng, hh, static_cast<const uint8_t*>(host_diff), len, logname);
  return MTC_OK;
}

int mtc_write_restart_log(const mtc_dedup_t* h, uint32_t select_chkpt, const char* logname) {
  if (!h || !logname) return ret(MTC_EINVAL, "NULL argument");
  mtc::write_restart_log(*h->eng, select_chkpt, logname);
  return MTC_OK;
}

int mtc_hash_chunks(int hash, const void* dev_data, uint64_t len, uint32_t chunk_size, void* dev_digests,
                    void* cuda_stream) {
  if (!dev_data || !dev_digests || chunk_size == 0) return ret(MTC_EINVAL, "bad argument");
  if (hash != MTC_HASH_MURMUR3 && hash != MTC_HASH_MD5) return ret(MTC_EINVAL, "unknown hash");
  if (len == 0) return MTC_OK;
  const uint64_t n = (len + chunk_size - 1) / chunk_size;
  if (n >= (1ull << 31)) return ret(MTC_ENOTSUP, "more than 2^31 chunks");
  mtc::LeafArgs a;
  a.data = static_cast<const uint8_t*>(dev_data);
  a.len = len;
  a.cs = chunk_size;
  a.n_chunks = (uint32_t)n;
  a.out = static_cast<mtc::Digest*>(dev_digests);
  a.hash_kind = hash;
  a.epi = mtc::EPI_HASH;
  mtc::TmaCache cache;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
  // a device error word for the call (a bounded wait that runs out sets it):
  // one per host thread and device, allocated on the thread's first call and
  // kept (an allocation per call would go through the default memory pool,
  // whose release at every synchronisation maps and unmaps device memory)
  thread_local uint32_t* tl_err[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return ret(MTC_ENOTSUP, "device ordinal above 63");
  cudaError_t e = cudaSuccess;
  if (!tl_err[dev]) e = cudaMalloc(reinterpret_cast<void**>(&tl_err[dev]), sizeof(uint32_t));
  uint32_t* err = e == cudaSuccess ? tl_err[dev] : nullptr;
  uint32_t err_host = 0;
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(uint32_t), s);
  a.err = err;
  if (e == cudaSuccess) e = mtc::launch_leaves(a, &cache, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err_host, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return ret(e == cudaErrorMemoryAllocation ? MTC_ENOMEM : MTC_ECUDA, cudaGetErrorString(e));
  if (err_host & mtc::DERR_SPIN) return ret(MTC_ETIMEOUT, "bounded device wait expired");
  return MTC_OK;
}

int mtc_digest_host(int hash, const void* host_data, uint64_t len, uint8_t out[16]) {
  if ((!host_data && len) || !out) return ret(MTC_EINVAL, "NULL argument");
  if (hash != MTC_HASH_MURMUR3 && hash != MTC_HASH_MD5) return ret(MTC_EINVAL, "unknown hash");
  mtc::digest_host(hash, static_cast<const uint8_t*>(host_data), len, out);
  return MTC_OK;
}

int mtc_digest_hex(const uint8_t d[16], char out[37]) {
  if (!d || !out) return ret(MTC_EINVAL, "NULL argument");
  static const char hx[] = "0123456789ABCDEF";
  char* c = out;
  for (int k = 0; k < 16; k++) {
    *c++ = hx[d[k] >> 4];
    *c++ = hx[d[k] & 15];
    if (k % 4 == 3) *c++ = ' ';
  }
  *c = 0;
  return MTC_OK;
}

// ---- batch ----
int mtc_batch_create(uint32_t n, const int* approaches, const int* hashes, const uint32_t* chunk_sizes,
                     mtc_batch_t** out) {
  if (!out) return ret(MTC_EINVAL, "out is NULL");
  *out = nullptr;
  if (n == 0 || !approaches || !hashes || !chunk_sizes) return ret(MTC_EINVAL, "empty or NULL member list");
  for (uint32_t i = 0; i < n; i++) {
    if (!valid_mode(approaches[i])) return ret(MTC_EINVAL, "unknown approach for member " + std::to_string(i));
    if (hashes[i] != MTC_HASH_MURMUR3 && hashes[i] != MTC_HASH_MD5)
      return ret(MTC_EINVAL, "unknown hash for member " + std::to_string(i));
    if (chunk_sizes[i] == 0) return ret(MTC_EINVAL, "chunk size 0 for member " + std::to_string(i));
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ret(MTC_ECUDA, "no CUDA device");
  auto* b = new (std::nothrow) mtc_batch;
  if (!b) return ret(MTC_ENOMEM, "out of host memory");
  b->b = new (std::nothrow) mtc::Batch();
  if (!b->b) { delete b; return ret(MTC_ENOMEM, "out of host memory"); }
  for (uint32_t i = 0; i < n; i++) {
    if (b->b->add(approaches[i], hashes[i], chunk_sizes[i]) < 0) {
      delete b->b;
      delete b;
      return ret(MTC_ECUDA, "cannot create a member stream");
    }
  }
  b->members.resize(n);
  for (uint32_t i = 0; i < n; i++) b->members[i] = mtc_dedup{b->b->member(i), true};
  *out = b;
  return MTC_OK;
}

int mtc_batch_destroy(mtc_batch_t* b) {
  if (!b) return MTC_OK;
  delete b->b;
  delete b;
  return MTC_OK;
}

int mtc_batch_member(mtc_batch_t* b, uint32_t i, mtc_dedup_t** member) {
  if (!b || !member) return ret(MTC_EINVAL, "NULL argument");
  if (i >= b->members.size()) return ret(MTC_EINVAL, "member index out of range");
  *member = &b->members[i];
  return MTC_OK;
}

int mtc_batch_checkpoint(mtc_batch_t* b, const void* const* dev_data, const uint64_t* lens, int make_baseline,
                         uint64_t* diff_lens) {
  if (!b || !dev_data || !lens) return ret(MTC_EINVAL, "NULL argument");
  int rc = b->b->checkpoint(reinterpret_cast<const uint8_t* const*>(dev_data), lens, make_baseline != 0, diff_lens);
  return rc ? ret(rc, b->b->last_error) : MTC_OK;
}

int mtc_batch_set_options(mtc_batch_t* b, int use_graph, uint32_t id_headroom) {
  if (!b) return ret(MTC_EINVAL, "NULL batch");
  b->b->set_use_graph(use_graph != 0);
  b->b->set_id_headroom(id_headroom);
  return MTC_OK;
}

int mtc_batch_get_info(const mtc_batch_t* b, mtc_batch_info_t* o) {
  if (!b || !o) return ret(MTC_EINVAL, "NULL argument");
  const mtc::BatchStats& s = b->b->stats();
  std::memset(o, 0, sizeof(*o));
  o->steps = s.steps;
  o->graph_captures = s.captures;
  o->graph_nodes = s.graph_nodes;
  o->kernels_per_step = s.kernels_per_step;
  o->last_device_ms = s.last_device_ms;
  o->last_call_ms = s.last_call_ms;
  for (int k = 0; k < 5; k++) o->host_ms[k] = s.host_ms[k];
  o->last_used_graph = s.last_used_graph;
  o->batched_leaf_members = s.last_used_graph ? s.batched_leaf_members : 0;
  return MTC_OK;
}

int mtc_batch_reserve(mtc_batch_t* b, const uint64_t* lens, uint64_t* bytes) {
  if (!b || !lens) return ret(MTC_EINVAL, "NULL argument");
  const int rc = b->b->reserve(lens, bytes);
  if (rc) return ret(rc, b->b->last_error);
  return MTC_OK;
}

int mtc_batch_autotune(mtc_batch_t* b, const uint64_t* lens) {
  if (!b || !lens) return ret(MTC_EINVAL, "NULL argument");
  for (uint32_t i = 0; i < b->b->size(); i++) {
    mtc::Engine* e = b->b->member(i);
    mtc::TuneResult r;
    std::string err;
    // members above 64 MiB share one 64 MiB trial (they fill every SM)
    const uint64_t trial = lens[i] < (64ull << 20) ? lens[i] : (64ull << 20);
    int rc = mtc::autotune(e->mode(), e->hash_kind(), e->chunk_size(), trial, true, &r, &err);
    if (rc) return ret(rc, err);
    e->set_leaf_tune(r.leaf);
    e->set_max_load(r.max_load);
  }
  return MTC_OK;
}

// ---- server ----
int mtc_server_create(const mtc_server_options_t* opt, mtc_server_t** out) {
  if (!out) return ret(MTC_EINVAL, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return ret(MTC_ECUDA, "no CUDA device");
  mtc::ServerOptions o;
  if (opt) {
    if (opt->hbm_budget) o.hbm_budget = opt->hbm_budget;
    if (opt->max_inflight) o.max_inflight = opt->max_inflight;
    if (opt->id_headroom) o.id_headroom = opt->id_headroom;
    o.use_graph = opt->use_graph;
    o.reserve_hbm = opt->reserve_hbm;
    o.pinned_reserve = opt->pinned_reserve;
  }
  auto* h = new (std::nothrow) mtc_server;
  if (!h) return ret(MTC_ENOMEM, "out of host memory");
  h->s = new (std::nothrow) mtc::Server(o);
  if (!h->s) { delete h; return ret(MTC_ENOMEM, "out of host memory"); }
  *out = h;
  return MTC_OK;
}

int mtc_server_destroy(mtc_server_t* s) {
  if (!s) return MTC_OK;
  s->s->drain(1e12);
  delete s->s;
  delete s;
  return MTC_OK;
}

int mtc_server_add_process(mtc_server_t* s, int approach, int hash, uint32_t chunk_size, uint32_t* pid) {
  if (!s || !pid) return ret(MTC_EINVAL, "NULL argument");
  if (!valid_mode(approach)) return ret(MTC_EINVAL, "unknown approach");
  if (hash != MTC_HASH_MURMUR3 && hash != MTC_HASH_MD5) return ret(MTC_EINVAL, "unknown hash");
  if (chunk_size == 0) return ret(MTC_EINVAL, "chunk size is 0");
  int rc = s->s->add_process(approach, hash, chunk_size, pid);
  return rc ? ret(rc, s->s->error()) : MTC_OK;
}

int mtc_server_submit_checkpoint(mtc_server_t* s, uint32_t pid, const void* dev_data, uint64_t len,
                                 int make_baseline, uint64_t* ticket) {
  if (!s) return ret(MTC_EINVAL, "NULL server");
  int rc = s->s->submit_checkpoint(pid, static_cast<const uint8_t*>(dev_data), len, make_baseline != 0, ticket);
  return rc ? ret(rc, s->s->error()) : MTC_OK;
}

int mtc_server_submit_restart(mtc_server_t* s, uint32_t pid, uint32_t chkpt_id, void* dev_out, uint64_t len,
                              uint64_t* ticket) {
  if (!s) return ret(MTC_EINVAL, "NULL server");
  int rc = s->s->submit_restart(pid, chkpt_id, static_cast<uint8_t*>(dev_out), len, ticket);
  return rc ? ret(rc, s->s->error()) : MTC_OK;
}

int mtc_server_poll(mtc_server_t* s, mtc_completion_t* out, uint32_t max, uint32_t* n, double wait_ms) {
  if (!s || !n || (max && !out)) return ret(MTC_EINVAL, "NULL argument");
  static_assert(sizeof(mtc_completion_t) == sizeof(mtc::Completion), "completion layout");
  *n = s->s->poll(reinterpret_cast<mtc::Completion*>(out), max, wait_ms);
  return MTC_OK;
}

int mtc_server_drain(mtc_server_t* s, double timeout_ms) {
  if (!s) return ret(MTC_EINVAL, "NULL server");
  return s->s->drain(timeout_ms) ? MTC_OK : ret(MTC_ETIMEOUT, "requests still in flight");
}

int mtc_server_chain_length(mtc_server_t* s, uint32_t pid, uint32_t* n) {
  if (!s || !n) return ret(MTC_EINVAL, "NULL argument");
  return s->s->chain_length(pid, n) ? ret(MTC_EINVAL, "unknown process") : MTC_OK;
}

int mtc_server_copy_diff(mtc_server_t* s, uint32_t pid, uint32_t chkpt_id, void* host, uint64_t capacity,
                         uint64_t* len) {
  if (!s) return ret(MTC_EINVAL, "NULL server");
  int rc = s->s->copy_diff(pid, chkpt_id, host, capacity, len);
  return rc ? ret(rc, "unknown process or checkpoint, or short buffer") : MTC_OK;
}

int mtc_server_get_stats(mtc_server_t* s, mtc_server_stats_t* o) {
  if (!s || !o) return ret(MTC_EINVAL, "NULL argument");
  const mtc::ServerStats t = s->s->stats();
  std::memset(o, 0, sizeof(*o));
  o->submitted = t.submitted; o->completed = t.completed; o->failed = t.failed;
  o->checkpoints = t.checkpoints; o->restarts = t.restarts;
  o->bytes_checkpointed = t.bytes_checkpointed; o->bytes_restarted = t.bytes_restarted;
  o->spilled_diffs = t.spilled_diffs; o->spilled_states = t.spilled_states; o->restored_states = t.restored_states;
  o->staged_diffs = t.staged_diffs; o->spilled_bytes = t.spilled_bytes;
  o->graph_captures = t.graph_captures; o->graph_replays = t.graph_replays;
  o->hbm_used = t.hbm_used; o->hbm_peak = t.hbm_peak; o->pinned_reserved = t.pinned_reserved;
  o->deferred_admissions = t.deferred_admissions; o->inflight_peak = t.inflight_peak;
  o->pinned_sync_grows = (uint32_t)t.pinned_sync_grows;
  o->pool_reserved_high = t.pool_reserved_high;
  o->pool_used_high = t.pool_used_high;
  for (int k = 0; k < 4; k++) o->worker_ms[k] = t.worker_ms[k];
  for (int k = 0; k < 3; k++) o->worker_max_ms[k] = t.worker_max_ms[k];
  return MTC_OK;
}

double mtc_now_ms(void) { return mtc::Server::now_ms(); }

// ---- tuning ----
int mtc_set_tuning(mtc_dedup_t* h, const mtc_tune_t* t) {
  if (!h || !t) return ret(MTC_EINVAL, "NULL argument");
  if (t->rows != 128 && t->rows != 256) return ret(MTC_EINVAL, "rows must be 128 or 256");
  if (t->ctas_per_sm < 0 || t->ctas_per_sm > 8) return ret(MTC_EINVAL, "ctas_per_sm out of range");
  if (!(t->max_load > 0.1 && t->max_load <= 0.95)) return ret(MTC_EINVAL, "max_load outside (0.1, 0.95]");
  if (t->threads_per_chunk != 0 && t->threads_per_chunk != 1 && t->threads_per_chunk != 32)
    return ret(MTC_EINVAL, "threads_per_chunk must be 1 or 32");
  h->eng->set_leaf_tune(mtc::LeafTune{t->rows, t->ctas_per_sm, t->direct ? 1 : 0,
                                      t->threads_per_chunk == 32 ? 32 : 1});
  h->eng->set_max_load(t->max_load);
  h->eng->set_own_graph(t->eager == 0);
  h->eng->set_untimed(t->untimed != 0);
  return MTC_OK;
}

int mtc_get_tuning(const mtc_dedup_t* h, mtc_tune_t* o) {
  if (!h || !o) return ret(MTC_EINVAL, "NULL argument");
  std::memset(o, 0, sizeof(*o));
  const mtc::LeafTune& t = h->eng->leaf_tune();
  o->rows = t.rows;
  o->ctas_per_sm = t.ctas_per_sm;
  o->direct = t.direct;
  o->threads_per_chunk = t.threads_per_chunk;
  o->eager = h->eng->own_graph() ? 0 : 1;
  o->untimed = h->eng->untimed() ? 1 : 0;
  o->max_load = h->eng->max_load();
  return MTC_OK;
}

int mtc_autotune(int approach, int hash, uint32_t chunk_size, uint64_t len, mtc_tune_t* best, double* best_ms,
                 double* default_ms) {
  if (!best) return ret(MTC_EINVAL, "NULL argument");
  if (!valid_mode(approach)) return ret(MTC_EINVAL, "unknown approach");
  if (hash != MTC_HASH_MURMUR3 && hash != MTC_HASH_MD5) return ret(MTC_EINVAL, "unknown hash");
  if (chunk_size == 0 || len == 0) return ret(MTC_EINVAL, "empty buffer or chunk size 0");
  mtc::TuneResult r;
  std::string err;
  int rc = mtc::autotune(approach, hash, chunk_size, len, false, &r, &err);
  if (rc) return ret(rc, err);
  std::memset(best, 0, sizeof(*best));
  best->rows = r.leaf.rows;
  best->ctas_per_sm = r.leaf.ctas_per_sm;
  best->direct = r.leaf.direct;
  best->threads_per_chunk = r.leaf.threads_per_chunk;
  best->max_load = r.max_load;
  if (best_ms) *best_ms = r.ms;
  if (default_ms) *default_ms = r.default_ms;
  return MTC_OK;
}

uint64_t mtc_launch_count(void) { return mtc::launch_count(); }

const char* mtc_last_error(void) { return t_err; }

}  // extern "C"
