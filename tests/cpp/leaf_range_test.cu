// The closed-form leaf_range of mtc_common.cuh against the reference's loop
// (include/kokkos_merkle_tree.hpp:102-142, restated below): every node of
// every tree with up to 2^14 nodes, then random nodes of random trees up to
// 2^31 nodes.  Host code only; prints "ok <count>" or the first mismatch.
#include <cstdint>
#include <cstdio>
#include <random>

#include "mtc_common.cuh"

static void reference_loop(uint32_t node, uint32_t num_nodes, uint32_t& lo, uint32_t& hi) {
  uint32_t l = 2 * node + 1, r = 2 * node + 2;
  while (l < num_nodes) { l = 2 * l + 1; r = 2 * r + 2; }
  l = (l - 1) / 2;
  r = (r - 2) / 2;
  if (r > num_nodes) r = num_nodes - 1;
  lo = l;
  hi = r;
}

static bool same(uint32_t node, uint32_t m) {
  uint32_t a, b, c, d;
  reference_loop(node, m, a, b);
  mtc::leaf_range(node, m, c, d);
  if (a == c && b == d) return true;
  std::printf("mismatch num_nodes=%u node=%u loop=[%u,%u] closed=[%u,%u]\n", m, node, a, b, c, d);
  return false;
}

int main() {
  unsigned long long n = 0;
  for (uint32_t m = 1; m <= (1u << 14); m++)
    for (uint32_t node = 0; node < m; node++, n++)
      if (!same(node, m)) return 1;
  std::mt19937_64 g(12345);
  for (int t = 0; t < 5000000; t++, n++) {
    const uint32_t m = 1 + (uint32_t)(g() % ((1u << 31) - 1));
    if (!same((uint32_t)(g() % m), m)) return 1;
  }
  std::printf("ok %llu\n", n);
  return 0;
}
