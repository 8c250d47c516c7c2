// host_digest.hpp -- calculate_digest_host (include/hash_functions.hpp:65-82):
// the digest of a whole host buffer, used to verify a restart.
#pragma once
#include <cstdint>

namespace mtc {
void digest_host(int hash_kind, const uint8_t* data, uint64_t len, uint8_t out[16]);
}
