// host_digest.cu -- whole-buffer digest on the host (calculate_digest_host,
// include/hash_functions.hpp:65-82).  Murmur3 is a serial chain over the whole
// buffer, so this stays on the CPU like the reference's.
#include <climits>
#include <cstring>

#include "host_digest.hpp"
#include "mtc_common.cuh"

namespace mtc {

static inline uint32_t ld32(const uint8_t* p) { uint32_t v; std::memcpy(&v, p, 4); return v; }

void digest_host(int kind, const uint8_t* p, uint64_t len, uint8_t out[16]) {
  Digest d;
  if (kind == HASH_MD5) {
    // Above INT_MAX bytes the reference feeds 128-byte pieces and replaces the
    // last piece by len % 128 bytes (include/kokkos_md5.hpp:293-301); the bytes
    // that reach MD5 are then exactly the first len - 128.
    uint64_t n = len > (uint64_t)INT_MAX ? len - 128 : len;
    Md5State s; s.init();
    uint32_t X[16];
    uint64_t off = 0;
    for (; off + 64 <= n; off += 64) {
      for (int i = 0; i < 16; i++) X[i] = ld32(p + off + 4 * i);
      s.block(X);
    }
    uint8_t tail[64] = {0};
    std::memcpy(tail, p + off, (size_t)(n - off));
    for (int i = 0; i < 16; i++) X[i] = ld32(tail + 4 * i);
    d = s.finish(X, (uint32_t)(n - off), n);
  } else {
    Murmur3State s; s.init();
    uint64_t off = 0;
    for (; off + 16 <= len; off += 16) s.block(ld32(p + off), ld32(p + off + 4), ld32(p + off + 8), ld32(p + off + 12));
    uint8_t tail[16] = {0};
    std::memcpy(tail, p + off, (size_t)(len - off));
    uint64_t t0, t1;
    std::memcpy(&t0, tail, 8);
    std::memcpy(&t1, tail + 8, 8);
    s.tail(t0, t1, (unsigned)(len - off));
    d = s.finish(len);
  }
  std::memcpy(out, d.w, 16);
}

}  // namespace mtc
