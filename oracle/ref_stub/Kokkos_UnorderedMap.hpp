// Declaration-only stand-in: include/map_helpers.hpp names
// Kokkos::UnorderedMap in type aliases; the hash headers never instantiate it.
#pragma once
#include "Kokkos_Core.hpp"
namespace Kokkos {
template <class K, class V, class D = DefaultExecutionSpace, class H = void, class E = void>
class UnorderedMap;
}
