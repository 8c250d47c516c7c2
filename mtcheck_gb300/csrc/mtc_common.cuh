// mtc_common.cuh -- device-side building blocks shared by every kernel of the
// deduplicator: the two digest functions, the digest -> NodeID open-addressing
// map, the Merkle-tree index arithmetic and the device error word.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mtc {

// Label values of the reference (include/utils.hpp:51-57).
enum : uint8_t { FIRST_OCUR = 0, FIXED_DUPL = 1, SHIFT_DUPL = 2, FIRST_DUPL = 3, DONE = 4 };
// Root flags written by the forest passes.
enum : uint8_t { ROOT_NONE = 0, ROOT_FO = 1, ROOT_SHIFT = 2 };
enum : int { HASH_MURMUR3 = 0, HASH_MD5 = 1 };

// Bits of the per-handle device error word.
enum : uint32_t {
  DERR_MAP_FULL = 1u << 0,      // probe sequence wrapped: table full
  DERR_SPIN = 1u << 1,          // a bounded device wait ran out
  DERR_FO_MISMATCH = 1u << 2,   // a first-occurrence root is not its digest's owner
  DERR_CAPACITY = 1u << 3,      // diff larger than the device staging buffer
  DERR_MISSING = 1u << 4,       // a root digest is absent from the map
  DERR_RANGE = 1u << 5,         // restart metadata out of range
  DERR_INTERIOR = 1u << 6,      // restart provenance names an interior node
  DERR_SORTKEYS = 1u << 7,      // more distinct source checkpoints than the sort supports
};

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may be scheduled while its predecessor on the stream is
// finishing.  Every kernel of the checkpoint sequence starts here: it waits
// for the predecessor grid's completion and memory (a no-op without such a
// dependency) before touching anything, then lets its own successor be
// scheduled.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Raise bits in a device error word (a launch given none records nothing).
__device__ __forceinline__ void raise_err(uint32_t* err, uint32_t bits) {
  if (err) atomicOr(err, bits);
}

struct __align__(16) Digest { uint32_t w[4]; };

__device__ __forceinline__ bool digest_eq(const Digest& a, const Digest& b) {
  return ((a.w[0] ^ b.w[0]) | (a.w[1] ^ b.w[1]) | (a.w[2] ^ b.w[2]) | (a.w[3] ^ b.w[3])) == 0;
}
__device__ __forceinline__ Digest ld_digest(const Digest* p) {
  uint4 v = *reinterpret_cast<const uint4*>(p);
  return Digest{{v.x, v.y, v.z, v.w}};
}
__device__ __forceinline__ void st_digest(Digest* p, const Digest& d) {
  *reinterpret_cast<uint4*>(p) = make_uint4(d.w[0], d.w[1], d.w[2], d.w[3]);
}

// ---------------------------------------------------------------------------
// Murmur3 variant of the reference (include/kokkos_murmur3.hpp:213-292):
// MurmurHash3_x64_128 with seed 0 in which rotl64 returns uint32_t, so each
// rotated value is truncated to its low 32 bits before further use.
// ---------------------------------------------------------------------------
#define MTC_HD __host__ __device__ __forceinline__
struct Murmur3State {
  uint64_t h1, h2;
  MTC_HD void init() { h1 = 0; h2 = 0; }
  MTC_HD static uint32_t rotl_lo(uint64_t x, int r) {
    // low 32 bits of the 64-bit rotation
    return (uint32_t)((x << r) | (x >> (64 - r)));
  }
  // one 16-byte body block given as four little-endian words
  MTC_HD void block(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3) {
    const uint64_t c1 = 0x87c37b91114253d5ull, c2 = 0x4cf5ad432745937full;
    uint64_t k1 = ((uint64_t)w1 << 32) | w0;
    uint64_t k2 = ((uint64_t)w3 << 32) | w2;
    k1 *= c1; k1 = rotl_lo(k1, 31); k1 *= c2; h1 ^= k1;
    h1 = rotl_lo(h1, 27); h1 += h2; h1 = h1 * 5 + 0x52dce729;
    k2 *= c2; k2 = rotl_lo(k2, 33); k2 *= c1; h2 ^= k2;
    h2 = rotl_lo(h2, 31); h2 += h1; h2 = h2 * 5 + 0x38495ab5;
  }
  // tail of `rem` (1..15) bytes packed little-endian in t0 (bytes 0..7) and t1 (8..15)
  MTC_HD void tail(uint64_t t0, uint64_t t1, unsigned rem) {
    const uint64_t c1 = 0x87c37b91114253d5ull, c2 = 0x4cf5ad432745937full;
    if (rem > 8) {
      uint64_t k2 = t1; k2 *= c2; k2 = rotl_lo(k2, 33); k2 *= c1; h2 ^= k2;
    }
    if (rem > 0) {
      uint64_t k1 = t0; k1 *= c1; k1 = rotl_lo(k1, 31); k1 *= c2; h1 ^= k1;
    }
  }
  MTC_HD static uint64_t fmix64(uint64_t k) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33; return k;
  }
  MTC_HD Digest finish(uint64_t len) {
    uint64_t a = h1 ^ len, b = h2 ^ len;
    a += b; b += a;
    a = fmix64(a); b = fmix64(b);
    a += b; b += a;
    return Digest{{(uint32_t)a, (uint32_t)(a >> 32), (uint32_t)b, (uint32_t)(b >> 32)}};
  }
};

// ---------------------------------------------------------------------------
// MD5 (RFC 1321) as computed by the reference for inputs of at most INT_MAX
// bytes (include/kokkos_md5.hpp:61-265).  Round constants are the RFC's
// floor(abs(sin(i+1)) * 2^32) table.
// ---------------------------------------------------------------------------
struct Md5State {
  uint32_t a, b, c, d;
  MTC_HD void init() { a = 0x67452301u; b = 0xefcdab89u; c = 0x98badcfeu; d = 0x10325476u; }
  MTC_HD static uint32_t rol(uint32_t x, int n) {
#ifdef __CUDA_ARCH__
    return __funnelshift_l(x, x, n);
#else
    return (x << n) | (x >> (32 - n));
#endif
  }
#define MTC_MD5_STEP(F, A, B, C, D, X, S, T) A = B + rol(A + (F) + (X) + (T), S)
  MTC_HD void block(const uint32_t* X) {
    uint32_t A = a, B = b, C = c, D = d;
#define F1(x, y, z) ((z) ^ ((x) & ((y) ^ (z))))
#define F2(x, y, z) ((y) ^ ((z) & ((x) ^ (y))))
#define F3(x, y, z) ((x) ^ (y) ^ (z))
#define F4(x, y, z) ((y) ^ ((x) | ~(z)))
    MTC_MD5_STEP(F1(B,C,D), A, B, C, D, X[0], 7, 0xd76aa478u);  MTC_MD5_STEP(F1(A,B,C), D, A, B, C, X[1], 12, 0xe8c7b756u);
    MTC_MD5_STEP(F1(D,A,B), C, D, A, B, X[2], 17, 0x242070dbu); MTC_MD5_STEP(F1(C,D,A), B, C, D, A, X[3], 22, 0xc1bdceeeu);
    MTC_MD5_STEP(F1(B,C,D), A, B, C, D, X[4], 7, 0xf57c0fafu);  MTC_MD5_STEP(F1(A,B,C), D, A, B, C, X[5], 12, 0x4787c62au);
    MTC_MD5_STEP(F1(D,A,B), C, D, A, B, X[6], 17, 0xa8304613u); MTC_MD5_STEP(F1(C,D,A), B, C, D, A, X[7], 22, 0xfd469501u);
    MTC_MD5_STEP(F1(B,C,D), A, B, C, D, X[8], 7, 0x698098d8u);  MTC_MD5_STEP(F1(A,B,C), D, A, B, C, X[9], 12, 0x8b44f7afu);
    MTC_MD5_STEP(F1(D,A,B), C, D, A, B, X[10], 17, 0xffff5bb1u); MTC_MD5_STEP(F1(C,D,A), B, C, D, A, X[11], 22, 0x895cd7beu);
    MTC_MD5_STEP(F1(B,C,D), A, B, C, D, X[12], 7, 0x6b901122u); MTC_MD5_STEP(F1(A,B,C), D, A, B, C, X[13], 12, 0xfd987193u);
    MTC_MD5_STEP(F1(D,A,B), C, D, A, B, X[14], 17, 0xa679438eu); MTC_MD5_STEP(F1(C,D,A), B, C, D, A, X[15], 22, 0x49b40821u);

    MTC_MD5_STEP(F2(B,C,D), A, B, C, D, X[1], 5, 0xf61e2562u);  MTC_MD5_STEP(F2(A,B,C), D, A, B, C, X[6], 9, 0xc040b340u);
    MTC_MD5_STEP(F2(D,A,B), C, D, A, B, X[11], 14, 0x265e5a51u); MTC_MD5_STEP(F2(C,D,A), B, C, D, A, X[0], 20, 0xe9b6c7aau);
    MTC_MD5_STEP(F2(B,C,D), A, B, C, D, X[5], 5, 0xd62f105du);  MTC_MD5_STEP(F2(A,B,C), D, A, B, C, X[10], 9, 0x02441453u);
    MTC_MD5_STEP(F2(D,A,B), C, D, A, B, X[15], 14, 0xd8a1e681u); MTC_MD5_STEP(F2(C,D,A), B, C, D, A, X[4], 20, 0xe7d3fbc8u);
    MTC_MD5_STEP(F2(B,C,D), A, B, C, D, X[9], 5, 0x21e1cde6u);  MTC_MD5_STEP(F2(A,B,C), D, A, B, C, X[14], 9, 0xc33707d6u);
    MTC_MD5_STEP(F2(D,A,B), C, D, A, B, X[3], 14, 0xf4d50d87u); MTC_MD5_STEP(F2(C,D,A), B, C, D, A, X[8], 20, 0x455a14edu);
    MTC_MD5_STEP(F2(B,C,D), A, B, C, D, X[13], 5, 0xa9e3e905u); MTC_MD5_STEP(F2(A,B,C), D, A, B, C, X[2], 9, 0xfcefa3f8u);
    MTC_MD5_STEP(F2(D,A,B), C, D, A, B, X[7], 14, 0x676f02d9u); MTC_MD5_STEP(F2(C,D,A), B, C, D, A, X[12], 20, 0x8d2a4c8au);

    MTC_MD5_STEP(F3(B,C,D), A, B, C, D, X[5], 4, 0xfffa3942u);  MTC_MD5_STEP(F3(A,B,C), D, A, B, C, X[8], 11, 0x8771f681u);
    MTC_MD5_STEP(F3(D,A,B), C, D, A, B, X[11], 16, 0x6d9d6122u); MTC_MD5_STEP(F3(C,D,A), B, C, D, A, X[14], 23, 0xfde5380cu);
    MTC_MD5_STEP(F3(B,C,D), A, B, C, D, X[1], 4, 0xa4beea44u);  MTC_MD5_STEP(F3(A,B,C), D, A, B, C, X[4], 11, 0x4bdecfa9u);
    MTC_MD5_STEP(F3(D,A,B), C, D, A, B, X[7], 16, 0xf6bb4b60u); MTC_MD5_STEP(F3(C,D,A), B, C, D, A, X[10], 23, 0xbebfbc70u);
    MTC_MD5_STEP(F3(B,C,D), A, B, C, D, X[13], 4, 0x289b7ec6u); MTC_MD5_STEP(F3(A,B,C), D, A, B, C, X[0], 11, 0xeaa127fau);
    MTC_MD5_STEP(F3(D,A,B), C, D, A, B, X[3], 16, 0xd4ef3085u); MTC_MD5_STEP(F3(C,D,A), B, C, D, A, X[6], 23, 0x04881d05u);
    MTC_MD5_STEP(F3(B,C,D), A, B, C, D, X[9], 4, 0xd9d4d039u);  MTC_MD5_STEP(F3(A,B,C), D, A, B, C, X[12], 11, 0xe6db99e5u);
    MTC_MD5_STEP(F3(D,A,B), C, D, A, B, X[15], 16, 0x1fa27cf8u); MTC_MD5_STEP(F3(C,D,A), B, C, D, A, X[2], 23, 0xc4ac5665u);

    MTC_MD5_STEP(F4(B,C,D), A, B, C, D, X[0], 6, 0xf4292244u);  MTC_MD5_STEP(F4(A,B,C), D, A, B, C, X[7], 10, 0x432aff97u);
    MTC_MD5_STEP(F4(D,A,B), C, D, A, B, X[14], 15, 0xab9423a7u); MTC_MD5_STEP(F4(C,D,A), B, C, D, A, X[5], 21, 0xfc93a039u);
    MTC_MD5_STEP(F4(B,C,D), A, B, C, D, X[12], 6, 0x655b59c3u); MTC_MD5_STEP(F4(A,B,C), D, A, B, C, X[3], 10, 0x8f0ccc92u);
    MTC_MD5_STEP(F4(D,A,B), C, D, A, B, X[10], 15, 0xffeff47du); MTC_MD5_STEP(F4(C,D,A), B, C, D, A, X[1], 21, 0x85845dd1u);
    MTC_MD5_STEP(F4(B,C,D), A, B, C, D, X[8], 6, 0x6fa87e4fu);  MTC_MD5_STEP(F4(A,B,C), D, A, B, C, X[15], 10, 0xfe2ce6e0u);
    MTC_MD5_STEP(F4(D,A,B), C, D, A, B, X[6], 15, 0xa3014314u); MTC_MD5_STEP(F4(C,D,A), B, C, D, A, X[13], 21, 0x4e0811a1u);
    MTC_MD5_STEP(F4(B,C,D), A, B, C, D, X[4], 6, 0xf7537e82u);  MTC_MD5_STEP(F4(A,B,C), D, A, B, C, X[11], 10, 0xbd3af235u);
    MTC_MD5_STEP(F4(D,A,B), C, D, A, B, X[2], 15, 0x2ad7d2bbu); MTC_MD5_STEP(F4(C,D,A), B, C, D, A, X[9], 21, 0xeb86d391u);
#undef F1
#undef F2
#undef F3
#undef F4
    a += A; b += B; c += C; d += D;
  }
#undef MTC_MD5_STEP
  // Final padding for a message of `len` bytes whose last `rem` (< 64) bytes
  // are in words tw[0..15] (zero beyond rem, little-endian).
  MTC_HD Digest finish(uint32_t* tw, uint32_t rem, uint64_t len) {
    // append 0x80 at byte `rem`
    tw[rem >> 2] |= 0x80u << (8 * (rem & 3));
    if (rem >= 56) {
      block(tw);
#pragma unroll
      for (int i = 0; i < 16; i++) tw[i] = 0;
    }
    uint64_t bits = len << 3;
    tw[14] = (uint32_t)bits; tw[15] = (uint32_t)(bits >> 32);
    block(tw);
    return Digest{{a, b, c, d}};
  }
};

// Digest of one 32-byte interior node: hash(left || right)
// (src/tree_approach.cpp:131, :221, :389, :459).
__device__ __forceinline__ Digest hash_pair(int kind, const Digest& l, const Digest& r) {
  if (kind == HASH_MD5) {
    Md5State s; s.init();
    uint32_t X[16] = {l.w[0], l.w[1], l.w[2], l.w[3], r.w[0], r.w[1], r.w[2], r.w[3], 0, 0, 0, 0, 0, 0, 0, 0};
    return s.finish(X, 32, 32);
  }
  Murmur3State s; s.init();
  s.block(l.w[0], l.w[1], l.w[2], l.w[3]);
  s.block(r.w[0], r.w[1], r.w[2], r.w[3]);
  return s.finish(32);
}

// Digest of `len` bytes at an arbitrary global address, one thread (any
// alignment; used for short, odd-sized and tail chunks).
__device__ __forceinline__ uint32_t ld_word_any(const uint8_t* p, uint64_t off, uint64_t len) {
  uint32_t w = 0;
#pragma unroll
  for (int b = 0; b < 4; b++) if (off + b < len) w |= (uint32_t)__ldg(p + off + b) << (8 * b);
  return w;
}
__device__ inline Digest hash_bytes(int kind, const uint8_t* p, uint64_t len) {
  const bool al4 = ((reinterpret_cast<uintptr_t>(p) & 3) == 0);
  auto word = [&](uint64_t off) -> uint32_t {
    if (al4 && off + 4 <= len) return __ldg(reinterpret_cast<const uint32_t*>(p + off));
    return ld_word_any(p, off, len);
  };
  if (kind == HASH_MD5) {
    Md5State s; s.init();
    uint32_t X[16];
    uint64_t off = 0;
    for (; off + 64 <= len; off += 64) {
#pragma unroll
      for (int i = 0; i < 16; i++) X[i] = word(off + 4 * i);
      s.block(X);
    }
#pragma unroll
    for (int i = 0; i < 16; i++) X[i] = word(off + 4 * i);
    return s.finish(X, (uint32_t)(len - off), len);
  }
  Murmur3State s; s.init();
  uint64_t off = 0;
  for (; off + 16 <= len; off += 16) s.block(word(off), word(off + 4), word(off + 8), word(off + 12));
  unsigned rem = (unsigned)(len - off);
  uint64_t t0 = ((uint64_t)word(off + 4) << 32) | word(off);
  uint64_t t1 = ((uint64_t)word(off + 12) << 32) | word(off + 8);
  s.tail(t0, t1, rem);
  return s.finish(len);
}

// Digest of `len` bytes held in a 4-byte aligned buffer that is zero from
// `len` up to the next 64-byte boundary (shared memory staging).
__device__ inline Digest hash_words(int kind, const uint32_t* w, uint32_t len) {
  if (kind == HASH_MD5) {
    Md5State s; s.init();
    uint32_t X[16];
    uint32_t off = 0;
    for (; off + 64 <= len; off += 64) {
#pragma unroll
      for (int i = 0; i < 16; i++) X[i] = w[off / 4 + i];
      s.block(X);
    }
#pragma unroll
    for (int i = 0; i < 16; i++) X[i] = w[off / 4 + i];
    return s.finish(X, len - off, len);
  }
  Murmur3State s; s.init();
  uint32_t off = 0;
  for (; off + 16 <= len; off += 16) s.block(w[off / 4], w[off / 4 + 1], w[off / 4 + 2], w[off / 4 + 3]);
  const uint64_t t0 = ((uint64_t)w[off / 4 + 1] << 32) | w[off / 4];
  const uint64_t t1 = ((uint64_t)w[off / 4 + 3] << 32) | w[off / 4 + 2];
  s.tail(t0, t1, len - off);
  return s.finish(len);
}

// ---------------------------------------------------------------------------
// Merkle heap index arithmetic, include/kokkos_merkle_tree.hpp:102-142
// (exact only for a power-of-two leaf count; restated as written).
// ---------------------------------------------------------------------------
// The reference descends from the node's children one level at a time until
// the left index passes num_nodes (l = 2l+1, r = 2r+2), then steps back one
// level.  After e doublings l = (node+1)*2^e - 1 and r = (node+2)*2^e - 2, so
// the same result follows from the smallest e >= 1 with (node+1)*2^e >=
// num_nodes+1, found from bit lengths; equal to the loop for every node of
// every tree size (checked exhaustively in tests).
__host__ __device__ __forceinline__ int bit_length64(uint64_t v) {
#ifdef __CUDA_ARCH__
  return 64 - __clzll((long long)v);
#else
  return v ? 64 - __builtin_clzll(v) : 0;
#endif
}
__host__ __device__ __forceinline__ void leaf_range(uint32_t node, uint32_t num_nodes, uint32_t& lo, uint32_t& hi) {
  const uint64_t a = (uint64_t)node + 1, b = (uint64_t)num_nodes + 1;
  int e = bit_length64(b) - bit_length64(a);
  if (e < 1) e = 1;
  if (e > 1 && (a << (e - 1)) >= b) e--;
  if ((a << e) < b) e++;
  uint64_t l = (a << (e - 1)) - 1, r = ((a + 1) << (e - 1)) - 2;
  if (r > num_nodes) r = (uint64_t)num_nodes - 1;
  lo = (uint32_t)l;
  hi = (uint32_t)r;
}
__host__ __device__ __forceinline__ uint32_t num_leaf_descendents(uint32_t node, uint32_t num_nodes) {
  uint32_t l, r; leaf_range(node, num_nodes, l, r); return r - l + 1;
}
__host__ __device__ __forceinline__ uint32_t leftmost_leaf(uint32_t node, uint32_t num_nodes) {
  uint32_t l, r; leaf_range(node, num_nodes, l, r); return l;
}

// ---------------------------------------------------------------------------
// Digest -> NodeID map (the reference's DigestNodeIDDeviceMap,
// include/map_helpers.hpp:105-110, with Kokkos::UnorderedMap's
// insert-if-absent semantics).  Open addressing, linear probing, 32-byte
// slots.  A slot is claimed by one 128-bit compare-and-swap of its key
// (all-ones = empty; a digest equal to that pattern is stored with its lowest
// bit cleared).  `win` packs (epoch << 38) | priority and starts all-ones;
// every insert of a key, its creator's included, applies atomicMin to it, so
//   * an entry created by an earlier launch (smaller epoch) is kept,
//   * among the inserts of one launch the lowest priority wins: the lowest
//     chunk or node (the reference's atomic_min), or the serial order of a
//     forest pass,
// and the old value an insert gets back tells whether the entry is older
// than its launch.  The node is win's low 32 bits.  `tree` (the checkpoint id
// of the first occurrence) is written by the creator and read by later
// launches; so is `first_chunk`, the chunk whose leaf insert created the
// entry (read by that checkpoint's demote pass).  No insert waits on another
// thread.
// ---------------------------------------------------------------------------
struct __align__(32) MapSlot {
  uint32_t key[4];
  unsigned long long win;
  uint32_t tree;
  uint32_t first_chunk;
};
struct DigestMap {
  MapSlot* slots;
  uint64_t mask;       // capacity - 1 (capacity a power of two)
  uint32_t* size;      // number of entries
};
constexpr unsigned long long kWinEmpty = ~0ull;
constexpr int kPrioBits = 38;
constexpr uint32_t kEpochLimit = 1u << (64 - kPrioBits);  // epochs are rebased to 0 before reaching it
constexpr int kMapFill = 0xff;                             // byte pattern of an empty table

__host__ __device__ __forceinline__ unsigned long long win_of(uint32_t epoch, uint64_t prio) {
  return ((unsigned long long)epoch << kPrioBits) | prio;
}
__host__ __device__ __forceinline__ uint32_t win_epoch(unsigned long long w) { return (uint32_t)(w >> kPrioBits); }
__host__ __device__ __forceinline__ uint32_t win_node(unsigned long long w) { return (uint32_t)w; }

enum : int { INS_FAILED = 0, INS_NEW = 1, INS_EXISTING = 2 };

__device__ __forceinline__ Digest map_key(const Digest& k) {
  Digest m = k;
  if ((k.w[0] & k.w[1] & k.w[2] & k.w[3]) == 0xffffffffu) m.w[0] = 0xfffffffeu;
  return m;
}
__device__ __forceinline__ bool key_empty(const uint4& v) { return (v.x & v.y & v.z & v.w) == 0xffffffffu; }
__device__ __forceinline__ bool key_eq(const uint4& v, const Digest& k) {
  return ((v.x ^ k.w[0]) | (v.y ^ k.w[1]) | (v.z ^ k.w[2]) | (v.w ^ k.w[3])) == 0;
}
__device__ __forceinline__ uint64_t slot_of(const Digest& k, uint64_t mask) {
  uint64_t a = ((uint64_t)k.w[1] << 32) | k.w[0];
  a ^= a >> 29; a *= 0xbf58476d1ce4e5b9ull; a ^= a >> 32;
  return a & mask;
}

// 128-bit compare-and-swap of a slot's key from empty to k; returns the key
// that was there (empty: the caller now owns the slot).
__device__ __forceinline__ uint4 claim_key(MapSlot* s, const Digest& k) {
  const unsigned long long e = ~0ull;
  const unsigned long long vlo = ((unsigned long long)k.w[1] << 32) | k.w[0];
  const unsigned long long vhi = ((unsigned long long)k.w[3] << 32) | k.w[2];
  unsigned long long olo, ohi;
  asm volatile(
      "{\n\t.reg .b128 c, v, o;\n\t"
      "mov.b128 c, {%2, %3};\n\t"
      "mov.b128 v, {%4, %5};\n\t"
      "atom.relaxed.gpu.global.cas.b128 o, [%6], c, v;\n\t"
      "mov.b128 {%0, %1}, o;\n\t}"
      : "=l"(olo), "=l"(ohi)
      : "l"(e), "l"(e), "l"(vlo), "l"(vhi), "l"(s->key)
      : "memory");
  return make_uint4((uint32_t)olo, (uint32_t)(olo >> 32), (uint32_t)ohi, (uint32_t)(ohi >> 32));
}

// atomicMin on an entry's win word, read first: win only decreases, so a
// value read at or below `w` (a stale read can only be higher than the
// current one) means the atomic would change nothing, and the read stands in
// for the value it would have returned: its epoch is the current one, and a
// node read too high only makes a caller lower it once more, which changes
// nothing either.
__device__ __forceinline__ unsigned long long win_min(unsigned long long* p, unsigned long long w) {
  const unsigned long long cur = __ldcg(p);
  return cur <= w ? cur : atomicMin(p, w);
}

// The slot of k, claimed if absent: INS_NEW (this thread created the entry),
// INS_EXISTING, or INS_FAILED (table full, error word set).
// A key, once claimed, never changes within a launch, so the slot is read
// before the compare-and-swap: a key that is already there (every duplicate
// of a digest, thousands of times over in a run of equal chunks) costs a
// load instead of an atomic on one contended line.  Only a read equal to k
// is taken as it is; anything else (another key, an empty slot, or a 16-byte
// read that saw half of a concurrent claim) goes through the atomic.
__device__ inline int map_claim(const DigestMap& m, const Digest& k, uint64_t* slot, uint32_t* err) {
  uint64_t i = slot_of(k, m.mask);
  for (uint64_t probe = 0; probe <= m.mask; probe++) {
    const uint4 seen = __ldcg(reinterpret_cast<const uint4*>(m.slots[i].key));
    if (key_eq(seen, k)) { *slot = i; return INS_EXISTING; }
    const uint4 old = claim_key(&m.slots[i], k);
    if (key_empty(old)) { *slot = i; return INS_NEW; }
    if (key_eq(old, k)) { *slot = i; return INS_EXISTING; }
    i = (i + 1) & m.mask;
  }
  raise_err(err, DERR_MAP_FULL);
  return INS_FAILED;
}

// Insert (k -> win, tree) with the priority rule above.  *old_win receives the
// entry's previous win: kWinEmpty for an entry created by this launch whose
// creator has not applied its own yet.  A new entry is not counted in
// m.size: the caller adds it (count_new_entries).
__device__ __forceinline__ int map_insert_win(const DigestMap& m, const Digest& k0, unsigned long long win,
                                              uint32_t tree, uint64_t* slot, unsigned long long* old_win,
                                              uint32_t* err) {
  const Digest k = map_key(k0);
  const int r = map_claim(m, k, slot, err);
  if (r == INS_FAILED) return r;
  MapSlot* s = &m.slots[*slot];
  if (r == INS_NEW) s->tree = tree;
  *old_win = win_min(&s->win, win);
  return r;
}

// Warp total of new entries added to m.size (every lane of the warp calls it).
__device__ __forceinline__ void count_new_entries(const DigestMap& m, uint32_t n) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(m.size, n);
}

// Slot index of key, or -1.  Plain loads: a key inserted by an earlier launch
// is found through slots that were all full when this launch started.
__device__ inline int64_t map_find(const DigestMap& m, const Digest& k0, uint32_t* err) {
  const Digest k = map_key(k0);
  uint64_t i = slot_of(k, m.mask);
  for (uint64_t probe = 0; probe <= m.mask; probe++) {
    const uint4 v = __ldcg(reinterpret_cast<const uint4*>(m.slots[i].key));
    if (key_empty(v)) return -1;
    if (key_eq(v, k)) return (int64_t)i;
    i = (i + 1) & m.mask;
  }
  return -1;
}

// Serial insertion order inside one forest pass: deeper levels first, then
// ascending node id.  Smaller key = inserted earlier = keeps the entry.
__device__ __forceinline__ uint64_t serial_prio(uint32_t node) {
  const uint32_t depth = 31 - __clz(node + 1);
  return ((uint64_t)(63 - depth) << 32) | node;
}
// Insert for a pass that spans several levels in one launch: an entry from an
// earlier launch is kept; among inserts of this pass the serially first wins.
// Returns 1 when the entry is new.
__device__ __forceinline__ uint32_t map_insert_serial(const DigestMap& m, const Digest& k, uint32_t node,
                                                      uint32_t tree, uint32_t epoch, uint32_t* err) {
  uint64_t slot;
  unsigned long long old;
  return map_insert_win(m, k, win_of(epoch, serial_prio(node)), tree, &slot, &old, err) == INS_NEW ? 1u : 0u;
}

// Plain read of a slot's value after the launch that wrote it has finished.
struct NodeIdDev { uint32_t node, tree; };
__device__ __forceinline__ NodeIdDev slot_value(const DigestMap& m, int64_t slot) {
  if (slot < 0) return NodeIdDev{0xffffffffu, 0xffffffffu};
  const MapSlot* s = &m.slots[slot];
  return NodeIdDev{win_node(s->win), s->tree};
}

}  // namespace mtc
