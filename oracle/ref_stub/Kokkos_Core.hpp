// Minimal stand-in for the two Kokkos function-attribute macros that the
// reference's hash headers (include/kokkos_murmur3.hpp, include/kokkos_md5.hpp,
// include/map_helpers.hpp) use.  It lets those headers compile on the host
// so that the oracle's digests can be pinned to the reference's own code.
// It provides no Kokkos functionality.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
namespace Kokkos {
struct DefaultExecutionSpace {};
struct DefaultHostExecutionSpace {};
}
