// Exposes the reference's own digest functions with C linkage so that tests
// can compare the oracle restatement against them.  Compiled by
// oracle/build.py directly from the reference's headers (include/
// kokkos_murmur3.hpp, include/kokkos_md5.hpp); output goes to oracle/_ref/.
// Test infrastructure only.
#include <climits>
#include "kokkos_murmur3.hpp"
#include "kokkos_md5.hpp"

extern "C" {
__attribute__((visibility("default"))) void ref_murmur3_hash(const void* data, uint64_t len, uint8_t* out) {
  kokkos_murmur3::hash(data, len, out);
}
__attribute__((visibility("default"))) void ref_md5_hash(const void* data, uint64_t len, uint8_t* out) {
  kokkos_md5::hash(data, len, out);
}
}
