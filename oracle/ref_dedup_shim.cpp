// Exposes the reference's own deduplicators (src/{tree,list,basic}_approach.cpp,
// compiled from where they lie against the serial Kokkos stand-in in
// oracle/kokkos_serial) with C linkage, so that tests can compare the
// oracle's restatement with the reference code itself: diff bytes of every
// checkpoint and restarted buffers.  The reference's hash() is Murmur3
// (include/hash_functions.hpp:17-20).  Test infrastructure only; output goes
// to oracle/_ref/ (oracle/build.py).
#include <cstring>
#include <vector>

#include "basic_approach.hpp"
#include "list_approach.hpp"
#include "tree_approach.hpp"

namespace {
BaseDeduplicator* make(int approach, uint32_t cs) {
  switch (approach) {
    case 2: return new BasicDeduplicator(cs);
    case 3: return new ListDeduplicator(cs);
    case 4: return new TreeDeduplicator(cs);
    default: return nullptr;
  }
}
}  // namespace

extern "C" {
__attribute__((visibility("default"))) void* refd_create(int approach, uint32_t chunk_size) {
  return make(approach, chunk_size);
}
__attribute__((visibility("default"))) void refd_destroy(void* h) { delete static_cast<BaseDeduplicator*>(h); }

// checkpoint(uint8_t*, size_t, HostMirror&, bool): the diff into a malloc'd
// buffer (release with refd_free); advances current_id like the reference
__attribute__((visibility("default"))) int refd_checkpoint(void* h, const uint8_t* data, uint64_t len,
                                                          int make_baseline, uint8_t** out, uint64_t* out_len) {
  auto* d = static_cast<BaseDeduplicator*>(h);
  Kokkos::View<uint8_t*>::HostMirror diff_h;
  d->checkpoint(const_cast<uint8_t*>(data), len, diff_h, make_baseline != 0);
  *out_len = diff_h.size();
  *out = static_cast<uint8_t*>(std::malloc(diff_h.size() ? diff_h.size() : 1));
  if (diff_h.size()) std::memcpy(*out, diff_h.data(), diff_h.size());
  return 0;
}
__attribute__((visibility("default"))) void refd_free(void* p) { std::free(p); }

// restart_chkpt(std::vector<HostMirror>&, int, View&) of a fresh deduplicator
// of the given approach into `out` (len bytes, the caller's fill kept where
// the reference writes nothing)
__attribute__((visibility("default"))) int refd_restart(int approach, uint32_t chunk_size, const uint8_t* const* diffs,
                                                       const uint64_t* lens, uint32_t n, uint32_t id, uint8_t* out,
                                                       uint64_t len) {
  std::vector<Kokkos::View<uint8_t*>::HostMirror> chain;
  for (uint32_t i = 0; i < n; i++) {
    Kokkos::View<uint8_t*>::HostMirror v("chkpt", lens[i]);
    std::memcpy(v.data(), diffs[i], lens[i]);
    chain.push_back(v);
  }
  Kokkos::View<uint8_t*> data(out, len);
  switch (approach) {
    case 2: BasicDeduplicator(chunk_size).restart_chkpt(chain, (int)id, data); break;
    case 3: ListDeduplicator(chunk_size).restart_chkpt(chain, (int)id, data); break;
    case 4: TreeDeduplicator(chunk_size).restart_chkpt(chain, (int)id, data); break;
    default: return 1;
  }
  return 0;
}
}
