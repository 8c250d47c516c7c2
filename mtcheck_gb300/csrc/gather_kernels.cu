// gather_kernels.cu -- everything between the leaf kernel and the finished
// incremental checkpoint in HBM:
//   * Merkle forest passes, several tree levels per launch (src/tree_approach.cpp
//     :124-227 baseline, :378-477 incremental; both incremental passes in
//     one traversal when no leaf was demoted);
//   * deterministic compaction of region roots in the order a serial backend
//     pushes them (replaces the atomic Vector::push, include/kokkos_vector.hpp:37-40);
//   * diff assembly: region sizes, repeat-count table, stable sort of the
//     shifted duplicates by source checkpoint, metadata and the chunk gather
//     (src/tree_approach.cpp:512-710, src/list_approach.cpp:79-247,
//     src/basic_approach.cpp:52-143).
#include <algorithm>
#include <cstdio>

#include "mtc_common.cuh"
#include "mtc_gather.hpp"
#include "mtc_scan.cuh"

namespace mtc {

namespace {

constexpr uint32_t kSortFastKeys = 1024;  // distinct source checkpoints per diff

inline uint32_t grid_for(uint64_t n, int threads, int per_sm = 8) {
  uint64_t g = (n + threads - 1) / threads;
  uint64_t cap = (uint64_t)num_sms() * per_sm;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return (uint32_t)g;
}

// ---------------------------------------------------------------------------
// Forest passes
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint8_t child_flag(uint8_t lab) {
  return (lab == FIXED_DUPL || lab == DONE) ? ROOT_NONE : (lab == SHIFT_DUPL ? ROOT_SHIFT : ROOT_FO);
}

// Several levels per launch: CTA b owns the subtree of interior node
// r = 2^d_top - 1 + b and computes its interior nodes from depth d_bot up to
// d_top.  Only the bottom children, leaves met on the way, digests and the
// results touch global memory.  pass 0: first-occurrence forest
// (src/tree_approach.cpp:378-404); pass 1: duplicate forest (:413-477), with
// baseline != 0 the baseline variant that tests the not-yet-hashed digest and
// then hashes and inserts every interior node (:155-227); pass 2: both
// incremental passes in one traversal (ForestArgs::fuse_gate).
constexpr uint32_t kSpanLevels = 9;     // 256 nodes on the bottom level of a span
constexpr uint32_t kBottomLevels = 12;  // bottom span: 16 leaves per thread, 4096 per block
constexpr uint32_t kBottomSink = 2048;  // queued inserts a bottom block holds in shared memory

// First-occurrence inserts are queued (node ids in ForestArgs::ins_queue) and
// issued by forest_insert_kernel after the pass's last launch: the
// first-occurrence pass never looks an entry up, the fused pass looks up only
// digests that no queued insert can equal, and the serial-order rule of
// map_insert_serial does not depend on arrival order.  A span block collects
// its ids in shared memory and appends them with one atomic.
struct IdSink {
  uint32_t* ids;  // shared memory
  uint32_t* n;    // shared counter
  uint32_t cap;   // ids beyond it go to the global queue directly
};
__device__ __forceinline__ void queue_insert(const ForestArgs& a, IdSink* sink, uint32_t n) {
  if (sink) {
    const uint32_t k = atomicAdd(sink->n, 1u);
    if (k < sink->cap) {
      sink->ids[k] = n;
      return;
    }
  }
  a.ins_queue[atomicAdd(a.ins_count, 1u)] = n;
}
__device__ __forceinline__ void flush_sink(const ForestArgs& a, const IdSink& sink, uint32_t* base) {
  __syncthreads();
  const uint32_t cnt = min(*sink.n, sink.cap);
  if (cnt == 0) return;
  if (threadIdx.x == 0) *base = atomicAdd(a.ins_count, cnt);
  __syncthreads();
  const uint32_t b = *base;
  for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) a.ins_queue[b + k] = sink.ids[k];
}

// One interior node n of a forest pass, given its children's labels: the
// hashing, map insert or lookup and children's root flags of the reference's
// level loops.  Writes n's label only when `store` is set (a span's top
// level, read by the next launch, or the baseline); only flags other than
// ROOT_NONE are written, the flag array being cleared before the first pass.
__device__ __forceinline__ uint8_t forest_node(const ForestArgs& a, int pass, int baseline, uint64_t n, uint8_t ll,
                                               uint8_t lr, uint32_t cur_id, uint32_t epoch_all, bool store) {
  const uint32_t l = 2 * (uint32_t)n + 1, rr = l + 1;
  uint8_t lab_n;
  if (pass == 0) {
    if (ll == FIRST_OCUR && lr == FIRST_OCUR) {
      lab_n = FIRST_OCUR;
      st_digest(a.tree + n, hash_pair(a.hash_kind, ld_digest(a.tree + l), ld_digest(a.tree + rr)));
      queue_insert(a, nullptr, (uint32_t)n);
    } else {
      lab_n = DONE;
    }
  } else {
    uint8_t fl = ROOT_NONE, fr = ROOT_NONE;
    if (ll != lr) {
      lab_n = DONE;
      fl = child_flag(ll);
      fr = child_flag(lr);
    } else if (ll == FIXED_DUPL) {
      lab_n = FIXED_DUPL;
    } else if (ll == SHIFT_DUPL) {
      Digest dg;
      if (baseline) {
        dg = ld_digest(a.tree + n);
      } else {
        dg = hash_pair(a.hash_kind, ld_digest(a.tree + l), ld_digest(a.tree + rr));
        st_digest(a.tree + n, dg);
      }
      if (map_find(a.map, dg, a.err) >= 0) {
        lab_n = SHIFT_DUPL;
      } else {
        lab_n = DONE;
        fl = ROOT_SHIFT;
        fr = ROOT_SHIFT;
      }
    } else if (ll == FIRST_OCUR) {
      lab_n = FIRST_OCUR;
      if (pass == 2) {
        st_digest(a.tree + n, hash_pair(a.hash_kind, ld_digest(a.tree + l), ld_digest(a.tree + rr)));
        queue_insert(a, nullptr, (uint32_t)n);
      }
    } else {
      lab_n = DONE;  // both first duplicates, or both done
    }
    if (fl != ROOT_NONE) a.rflag[canon_pos(a, l)] = fl;
    if (fr != ROOT_NONE) a.rflag[canon_pos(a, rr)] = fr;
    if (baseline) {
      Digest dg = hash_pair(a.hash_kind, ld_digest(a.tree + l), ld_digest(a.tree + rr));
      st_digest(a.tree + n, dg);
      if (map_insert_serial(a.map, dg, (uint32_t)n, cur_id, epoch_all, a.err)) atomicAdd(a.map.size, 1u);
    }
  }
  if (store) a.labels[n] = lab_n;
  return lab_n;
}

// Label of node n at a level of a span: final for a leaf (or DONE past the
// end), otherwise computed from the children's labels.
__device__ __forceinline__ uint8_t forest_label(const ForestArgs& a, int pass, int baseline, uint64_t n,
                                                uint64_t last_interior, uint64_t M, uint8_t ll, uint8_t lr,
                                                uint32_t cur_id, uint32_t epoch_all, bool store) {
  if (n > last_interior) return n < M ? a.labels[n] : DONE;
  return forest_node(a, pass, baseline, n, ll, lr, cur_id, epoch_all, store);
}

// Resolves the pass of an incremental launch: with the fuse gate open the
// first-occurrence launch runs both passes (2) and the duplicate launch has
// nothing left to do (-1).
__device__ __forceinline__ int resolve_pass(const ForestArgs& a, int pass) {
  if (a.fuse_gate && *a.fuse_gate == 0) return pass == 1 ? -1 : 2;
  return pass;
}

// Levels d_bot .. d_top of the subtree rooted at depth d_top, node labels in
// shared memory, one barrier per level.  Serves every span shape, and the
// baseline's duplicate pass, whose shift test must see every insert of the
// levels below it.
__global__ void __launch_bounds__(256) forest_span_kernel(ForestArgs a, int pass, int baseline, uint32_t N,
                                                          uint32_t d_top, uint32_t d_bot) {
  pdl_enter();
  __shared__ uint8_t lab[2][2 << (kSpanLevels - 1)];
  pass = resolve_pass(a, pass);
  if (pass < 0) return;
  const uint32_t cur_id = a.sp->cur, epoch_all = a.sp->epoch + 2;
  const uint64_t r = ((1ull << d_top) - 1) + blockIdx.x;
  const uint64_t last_interior = (uint64_t)N - 2, M = 2ull * N - 1;
  if (r > last_interior) return;
  const uint32_t wb = 1u << (d_bot - d_top);
  uint8_t* child = lab[0];
  uint8_t* cur = lab[1];
  {
    const uint64_t cfirst = (r + 1) * (2ull * wb) - 1;  // subtree nodes at depth d_bot + 1
    for (uint32_t i = threadIdx.x; i < 2 * wb; i += blockDim.x) {
      const uint64_t n = cfirst + i;
      child[i] = n < M ? a.labels[n] : DONE;
    }
  }
  __syncthreads();
  for (int d = (int)d_bot; d >= (int)d_top; d--) {
    const uint32_t width = 1u << (d - d_top);
    const uint64_t first = (r + 1) * width - 1;
    for (uint32_t i = threadIdx.x; i < width; i += blockDim.x)
      cur[i] = forest_label(a, pass, baseline, first + i, last_interior, M, child[2 * i], child[2 * i + 1], cur_id,
                            epoch_all, baseline || d == (int)d_top);
    __syncthreads();
    uint8_t* t = child;
    child = cur;
    cur = t;
  }
}

// Whether a node's digest is read by its parent in a pass: first-occurrence
// pairs are hashed in the first pass, shifted-duplicate pairs in the second,
// both in the fused pass 2.
__device__ __forceinline__ bool digest_wanted(int pass, uint8_t lab) {
  return pass == 0 ? lab == FIRST_OCUR : pass == 1 ? lab == SHIFT_DUPL : (lab == FIRST_OCUR || lab == SHIFT_DUPL);
}

// One interior node n of an incremental pass (first-occurrence forest
// src/tree_approach.cpp:378-404, duplicate forest :413-477, or both: pass 2)
// given its children's labels and digests; `dg` receives n's digest when n is
// hashed.  First-occurrence inserts go to the block's sink.
template <int HK>
__device__ __forceinline__ uint8_t span_node(const ForestArgs& a, int pass, uint32_t n, uint8_t ll, uint8_t lr,
                                             const Digest& dl, const Digest& dr, Digest& dg, bool store,
                                             IdSink* sink) {
  const uint32_t l = 2 * n + 1, rr = l + 1;
  uint8_t lab_n;
  if (pass == 0) {
    if (ll == FIRST_OCUR && lr == FIRST_OCUR) {
      lab_n = FIRST_OCUR;
      dg = hash_pair(HK, dl, dr);
      st_digest(a.tree + n, dg);
      queue_insert(a, sink, n);
    } else {
      lab_n = DONE;
    }
  } else {
    uint8_t fl = ROOT_NONE, fr = ROOT_NONE;
    if (ll != lr) {
      lab_n = DONE;
      fl = child_flag(ll);
      fr = child_flag(lr);
    } else if (ll == FIXED_DUPL) {
      lab_n = FIXED_DUPL;
    } else if (ll == SHIFT_DUPL) {
      dg = hash_pair(HK, dl, dr);
      st_digest(a.tree + n, dg);
      if (map_find(a.map, dg, a.err) >= 0) {
        lab_n = SHIFT_DUPL;
      } else {
        lab_n = DONE;
        fl = ROOT_SHIFT;
        fr = ROOT_SHIFT;
      }
    } else if (ll == FIRST_OCUR) {
      lab_n = FIRST_OCUR;
      if (pass == 2) {
        dg = hash_pair(HK, dl, dr);
        st_digest(a.tree + n, dg);
        queue_insert(a, sink, n);
      }
    } else {
      lab_n = DONE;  // both first duplicates, or both done
    }
    if (fl != ROOT_NONE) a.rflag[canon_pos(a, l)] = fl;
    if (fr != ROOT_NONE) a.rflag[canon_pos(a, rr)] = fr;
  }
  if (store) a.labels[n] = lab_n;
  return lab_n;
}

// Node n on the deepest interior level: a leaf there (a ragged last level)
// keeps its label and stored digest; an interior node is computed.
template <int HK>
__device__ __forceinline__ uint8_t span_label(const ForestArgs& a, int pass, uint64_t n, uint64_t last_interior,
                                              uint64_t M, uint8_t ll, uint8_t lr, const Digest& dl,
                                              const Digest& dr, Digest& dg, IdSink* sink) {
  if (n > last_interior) {
    const uint8_t lab = n < M ? a.labels[n] : DONE;
    if (digest_wanted(pass, lab)) dg = ld_digest(a.tree + n);
    return lab;
  }
  return span_node<HK>(a, pass, (uint32_t)n, ll, lr, dl, dr, dg, false, sink);
}

__device__ __forceinline__ Digest shfl_digest(const Digest& d, int src) {
  constexpr unsigned kFull = 0xffffffffu;
  return Digest{{__shfl_sync(kFull, d.w[0], src), __shfl_sync(kFull, d.w[1], src), __shfl_sync(kFull, d.w[2], src),
                 __shfl_sync(kFull, d.w[3], src)}};
}

// The eight upper levels of a span below node r, from one node per thread
// (relative depth 8, node (r+1)*256-1+threadIdx.x, label `lab`, digest `dg`):
// five inside each warp (children's labels and digests by shuffle), then
// three in warp 0 from the eight warps' results.  Stores r's label.  Every
// node here is interior.
template <int HK>
__device__ __forceinline__ void upper_levels(const ForestArgs& a, int pass, uint64_t r, uint8_t lab, Digest dg,
                                             IdSink* sink, uint8_t* top8, Digest* topdg) {
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr unsigned kFull = 0xffffffffu;
#pragma unroll 1
  for (uint32_t step = 1; step <= 5; step++) {
    const int sl = (2 * lane) & 31, sr = (2 * lane + 1) & 31;
    const uint8_t cl = (uint8_t)__shfl_sync(kFull, lab, sl);
    const uint8_t cr = (uint8_t)__shfl_sync(kFull, lab, sr);
    Digest dl{{0, 0, 0, 0}}, dr{{0, 0, 0, 0}};
    if (__any_sync(kFull, digest_wanted(pass, lab))) {
      dl = shfl_digest(dg, sl);
      dr = shfl_digest(dg, sr);
    }
    const uint32_t width = 32u >> step;
    if (lane < width) {
      const uint64_t n = (r + 1) * (256u >> step) - 1 + warp * width + lane;
      lab = span_node<HK>(a, pass, (uint32_t)n, cl, cr, dl, dr, dg, false, sink);
    }
  }
  if (lane == 0) {
    top8[warp] = lab;
    topdg[warp] = dg;
  }
  __syncthreads();
  if (warp == 0) {
    lab = lane < 8 ? top8[lane] : DONE;
    if (lane < 8) dg = topdg[lane];
#pragma unroll 1
    for (uint32_t step = 6; step <= 8; step++) {
      const int sl = (2 * lane) & 31, sr = (2 * lane + 1) & 31;
      const uint8_t cl = (uint8_t)__shfl_sync(kFull, lab, sl);
      const uint8_t cr = (uint8_t)__shfl_sync(kFull, lab, sr);
      const Digest dl = shfl_digest(dg, sl), dr = shfl_digest(dg, sr);
      const uint32_t width = 256u >> step;
      if (lane < width) {
        const uint64_t n = (r + 1) * width - 1 + lane;
        lab = span_node<HK>(a, pass, (uint32_t)n, cl, cr, dl, dr, dg, step == 8, sink);
      }
    }
  }
}

// A full span of 9 levels (256 nodes on its bottom level) for the incremental
// passes and the baseline's first-occurrence pass: the bottom nodes' children
// come from memory, the rest by upper_levels -- one block barrier instead of
// nine, and no digest goes through memory between levels (they are still
// stored: the tree keeps every digest for the next checkpoint).
template <int HK>
__global__ void __launch_bounds__(256) forest_span9_warp_kernel(ForestArgs a, int pass, uint32_t N, uint32_t d_top) {
  pdl_enter();
  __shared__ uint8_t top8[8];
  __shared__ Digest topdg[8];
  __shared__ uint32_t ids[(1u << kSpanLevels) - 1];  // one per interior node: never overflows
  __shared__ uint32_t ids_n, ids_base;
  const uint64_t r = ((1ull << d_top) - 1) + blockIdx.x;
  const uint64_t last_interior = (uint64_t)N - 2, M = 2ull * N - 1;
  if (r > last_interior) return;
  pass = resolve_pass(a, pass);
  if (pass < 0) return;
  if (threadIdx.x == 0) ids_n = 0;
  __syncthreads();
  IdSink sink{ids, &ids_n, (1u << kSpanLevels) - 1};
  uint8_t lab;
  Digest dg{{0, 0, 0, 0}};
  {
    const uint64_t n = (r + 1) * 256 - 1 + threadIdx.x;
    uint8_t ll = DONE, lr = DONE;
    Digest dl{{0, 0, 0, 0}}, dr{{0, 0, 0, 0}};
    if (n <= last_interior) {
      const uint64_t c = 2 * n + 1;
      ll = c < M ? a.labels[c] : DONE;
      lr = c + 1 < M ? a.labels[c + 1] : DONE;
      if (ll == lr && digest_wanted(pass, ll)) {
        dl = ld_digest(a.tree + c);
        dr = ld_digest(a.tree + c + 1);
      }
    }
    lab = span_label<HK>(a, pass, n, last_interior, M, ll, lr, dl, dr, dg, &sink);
  }
  upper_levels<HK>(a, pass, r, lab, dg, &sink, top8, topdg);
  if (pass != 1) flush_sink(a, sink, &ids_base);
}

// Byte-parallel labelling of four (left, right) pairs per 32-bit word, the
// rules of span_node: P receives the parents' labels, FL / FR the children's
// root flags (duplicate passes), XF the pairs to hash and insert
// (first-occurrence passes), XS the pairs to hash and look up (duplicate
// passes; their parents read SHIFT_DUPL until resolved).  Bytes are 0xff in
// the X masks.
constexpr uint32_t kB1 = 0x01010101u;
__device__ __forceinline__ uint32_t child_flags4(uint32_t x) {
  const uint32_t sh = __vcmpeq4(x, SHIFT_DUPL * kB1);
  const uint32_t none = __vcmpeq4(x, FIXED_DUPL * kB1) | __vcmpeq4(x, DONE * kB1);
  return (sh & (ROOT_SHIFT * kB1)) | (~sh & ~none & (ROOT_FO * kB1));
}
__device__ __forceinline__ void label_pairs4(int pass, uint32_t L, uint32_t R, uint32_t& P, uint32_t& FL,
                                             uint32_t& FR, uint32_t& XF, uint32_t& XS) {
  const uint32_t eq = __vcmpeq4(L, R);
  const uint32_t fo = eq & __vcmpeq4(L, FIRST_OCUR * kB1);
  P = (DONE * kB1) & ~fo;  // FIRST_OCUR is 0
  FL = FR = XS = 0;
  XF = pass != 1 ? fo : 0;
  if (pass != 0) {
    const uint32_t fix = eq & __vcmpeq4(L, FIXED_DUPL * kB1);
    const uint32_t sh = eq & __vcmpeq4(L, SHIFT_DUPL * kB1);
    P = (P & ~(fix | sh)) | (fix & (FIXED_DUPL * kB1)) | (sh & (SHIFT_DUPL * kB1));
    FL = ~eq & child_flags4(L);
    FR = ~eq & child_flags4(R);
    XS = sh;
  }
}
__device__ __forceinline__ void set_byte(uint32_t& w, int b, uint32_t v) {
  w = (w & ~(0xffu << (8 * b))) | (v << (8 * b));
}

// A thread's four levels below node (r+1)*256-1+t when its 8 nodes on the
// deepest interior level are all interior: the 16 children's labels in c[4]
// (byte j = child j).  Returns the label of the thread's top node and its
// digest in dg when a parent reads it.
template <int HK>
__device__ __forceinline__ uint8_t thread_levels_bytewise(const ForestArgs& a, int pass, uint64_t r, uint32_t t,
                                                          uint32_t c[4], IdSink* sink, Digest (*work)[256],
                                                          Digest& dg) {
  uint64_t nb = (r + 1) * 2048 - 1 + 8ull * t;  // first parent of the level
#pragma unroll 1
  for (int lvl = 0; lvl < 4; lvl++) {
    uint32_t P[2], FL[2], FR[2], XF[2], XS[2];
#pragma unroll
    for (int q = 0; q < 2; q++)
      label_pairs4(pass, __byte_perm(c[2 * q], c[2 * q + 1], 0x6420), __byte_perm(c[2 * q], c[2 * q + 1], 0x7531),
                   P[q], FL[q], FR[q], XF[q], XS[q]);
    // pairs that hash: ascending, so work[i] is written after its children
    // work[2i], work[2i+1] of the level below were read
#pragma unroll
    for (int q = 0; q < 2; q++) {
      uint32_t X = XF[q] | XS[q];
      while (X) {
        const int b = (__ffs(X) - 1) >> 3;
        X &= ~(0xffu << (8 * b));
        const uint32_t i = 4 * q + b;
        const uint64_t n = nb + i;
        Digest dl, dr;
        if (lvl == 0) {
          dl = ld_digest(a.tree + 2 * n + 1);
          dr = ld_digest(a.tree + 2 * n + 2);
        } else {
          dl = work[2 * i][t];
          dr = work[2 * i + 1][t];
        }
        const Digest d = hash_pair(HK, dl, dr);
        st_digest(a.tree + n, d);
        if ((XF[q] >> (8 * b)) & 1) {
          queue_insert(a, sink, (uint32_t)n);
          work[i][t] = d;
        } else if (map_find(a.map, d, a.err) >= 0) {
          work[i][t] = d;  // parent stays SHIFT_DUPL
        } else {
          set_byte(P[q], b, DONE);
          set_byte(FL[q], b, ROOT_SHIFT);
          set_byte(FR[q], b, ROOT_SHIFT);
        }
      }
    }
    // children's root flags, children in order at consecutive canonical positions
    if ((FL[0] | FR[0] | FL[1] | FR[1]) != 0) {
      const uint64_t cp0 = canon_pos(a, (uint32_t)(2 * nb + 1));
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const uint32_t f4[2] = {__byte_perm(FL[q], FR[q], 0x5140), __byte_perm(FL[q], FR[q], 0x7362)};
#pragma unroll
        for (int k = 0; k < 2; k++) {
          uint32_t f = f4[k];
          while (f) {
            const int b = (__ffs(f) - 1) >> 3;
            a.rflag[cp0 + 8 * q + 4 * k + b] = (uint8_t)(f >> (8 * b));
            f &= ~(0xffu << (8 * b));
          }
        }
      }
    }
    c[0] = P[0];
    c[1] = P[1];
    c[2] = c[3] = DONE * kB1;  // pairs past the level's width: DONE, no flags
    nb = (nb - 1) / 2;
  }
  const uint8_t lab = (uint8_t)c[0];
  if (digest_wanted(pass, lab)) dg = work[0][t];
  return lab;
}

// The bottom span of an incremental pass (and of the baseline's
// first-occurrence pass): 12 levels, 4096 leaves per block.  Each thread
// reads the labels of its 16 children with one aligned 16-byte load (the
// first byte comes from the lane before) and computes its 8, 4, 2 and 1 nodes
// in a loop, labels packed in a 64-bit word, digests in shared memory; a
// thread whose 16 children are all unchanged (fixed duplicates) has nothing
// to hash, flag or insert.  upper_levels does the rest.  Loops rather than
// unrolled levels keep the kernel small enough for the instruction cache.
template <int HK>
__global__ void __launch_bounds__(256) forest_bottom12_kernel(ForestArgs a, int pass, uint32_t N, uint32_t d_top) {
  pdl_enter();
  __shared__ uint8_t top8[8];
  __shared__ Digest topdg[8];
  __shared__ uint32_t ids[kBottomSink];
  __shared__ uint32_t ids_n, ids_base;
  __shared__ Digest work[8][256];  // [node of the thread's level][thread]: 16-byte lanes, no bank conflicts
  const uint64_t r = ((1ull << d_top) - 1) + blockIdx.x;
  const uint64_t last_interior = (uint64_t)N - 2, M = 2ull * N - 1;
  if (r > last_interior) return;
  pass = resolve_pass(a, pass);
  if (pass < 0) return;
  if (threadIdx.x == 0) ids_n = 0;
  __syncthreads();
  IdSink sink{ids, &ids_n, kBottomSink};
  const uint32_t t = threadIdx.x, lane = t & 31;
  constexpr unsigned kFull = 0xffffffffu;
  // children (relative depth 12) cb .. cb+15; cb + 1 is a multiple of 16
  const uint64_t cb = (r + 1) * 4096 - 1 + 16ull * t;
  uint4 v;
  if (cb + 17 <= M) {
    v = *reinterpret_cast<const uint4*>(a.labels + cb + 1);
  } else {
    uint32_t w[4] = {0, 0, 0, 0};
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const uint64_t c = cb + 1 + j;
      w[j >> 2] |= (uint32_t)(c < M ? a.labels[c] : DONE) << (8 * (j & 3));
    }
    v = make_uint4(w[0], w[1], w[2], w[3]);
  }
  uint32_t first = __shfl_up_sync(kFull, v.w, 1) >> 24;  // byte 15 of the lane before = child cb
  if (lane == 0) first = cb < M ? a.labels[cb] : DONE;
  // child j's label is byte j of (lo, hi)
  uint64_t lo = ((uint64_t)((v.y << 8) | (v.x >> 24)) << 32) | ((v.x << 8) | first);
  uint64_t hi = ((uint64_t)((v.w << 8) | (v.z >> 24)) << 32) | ((v.y >> 24) | (v.z << 8));
  const uint64_t nb1 = (r + 1) * 2048 - 1 + 8ull * t;  // relative depth 11: the deepest interior level
  uint8_t lab;
  Digest dg{{0, 0, 0, 0}};
  constexpr uint64_t kFixed8 = 0x0101010101010101ull * FIXED_DUPL;
  if (lo == kFixed8 && hi == kFixed8 && nb1 + 7 <= last_interior) {
    lab = pass == 0 ? DONE : FIXED_DUPL;
  } else if (nb1 + 7 <= last_interior) {
    uint32_t c[4] = {(uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32)};
    lab = thread_levels_bytewise<HK>(a, pass, r, t, c, &sink, work, dg);
  } else {
    uint64_t nb = nb1;
    uint32_t width = 8;
#pragma unroll 1
    for (int lvl = 0; lvl < 4; lvl++) {
      uint64_t out = 0;
#pragma unroll 1
      for (uint32_t i = 0; i < width; i++) {
        const uint32_t j = 2 * i;
        const uint8_t ll = (uint8_t)((j < 8 ? lo >> (8 * j) : hi >> (8 * (j - 8))) & 0xff);
        const uint8_t lr = (uint8_t)((j + 1 < 8 ? lo >> (8 * (j + 1)) : hi >> (8 * (j - 7))) & 0xff);
        const uint64_t n = nb + i;
        Digest dl{{0, 0, 0, 0}}, dr{{0, 0, 0, 0}}, d{{0, 0, 0, 0}};
        if (ll == lr && digest_wanted(pass, ll)) {
          if (lvl == 0) {
            if (n <= last_interior) {
              dl = ld_digest(a.tree + 2 * n + 1);
              dr = ld_digest(a.tree + 2 * n + 2);
            }
          } else {
            dl = work[j][t];
            dr = work[j + 1][t];
          }
        }
        const uint8_t l = lvl == 0 ? span_label<HK>(a, pass, n, last_interior, M, ll, lr, dl, dr, d, &sink)
                                   : span_node<HK>(a, pass, (uint32_t)n, ll, lr, dl, dr, d, false, &sink);
        if (digest_wanted(pass, l)) work[i][t] = d;  // read back only at the next level, from a higher index
        out |= (uint64_t)l << (8 * i);
        if (lvl == 3) dg = d;
      }
      lo = out;
      hi = 0;
      nb = (nb - 1) / 2;  // parent of the level's first node
      width >>= 1;
    }
    lab = (uint8_t)lo;
  }
  upper_levels<HK>(a, pass, r, lab, dg, &sink, top8, topdg);
  if (pass != 1) flush_sink(a, sink, &ids_base);
}

// The queued first-occurrence inserts of a pass, one thread per node, over
// blocks b0 .. b0+nb-1 of the launch.
__device__ __forceinline__ void drain_inserts(const ForestArgs& a, uint32_t b0, uint32_t nb) {
  const uint32_t n = *a.ins_count;
  const uint32_t cur_id = a.sp->cur, epoch_fo = a.sp->epoch + 1;
  uint32_t created = 0;
  for (uint32_t k = (blockIdx.x - b0) * blockDim.x + threadIdx.x; k < n; k += nb * blockDim.x) {
    const uint32_t node = a.ins_queue[k];
    created += map_insert_serial(a.map, ld_digest(a.tree + node), node, cur_id, epoch_fo, a.err);
  }
  count_new_entries(a.map, created);
}
__device__ __forceinline__ bool forest_fused(const ForestArgs& a) { return a.fuse_gate && *a.fuse_gate == 0; }

// After the first-occurrence pass: the duplicate pass that follows looks its
// digests up.  A fused pass looks nothing up that these inserts could add,
// so its inserts wait for the root count (root_count_kernel's extra blocks).
__global__ void forest_insert_kernel(ForestArgs a) {
  pdl_enter();
  if (forest_fused(a)) return;
  drain_inserts(a, 0, gridDim.x);
}

// ---------------------------------------------------------------------------
// Root compaction in serial push order.  rflag holds the flags at canonical
// positions, so the lists are a stable compaction of one byte array.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t node_at(const ForestArgs& a, uint64_t p) {
  if (a.ascending) return (uint32_t)p + 1;
  if (p < a.sizeD) return (uint32_t)(((1ull << a.D) - 1) + p);
  // levels D-1, D-2, ... follow with sizes 2^(D-1), 2^(D-2), ...: position q
  // past level D lies on level d with x = 2^D - q in (2^d, 2^(d+1)]
  const uint64_t x = (1ull << a.D) - (p - a.sizeD);
  const int d = 63 - __clzll((long long)(x - 1));
  return (uint32_t)(((1ull << d) - 1) + ((2ull << d) - x));
}

// 64 contiguous flags per thread (four 16-byte loads), 32 Ki flags per
// tile; counts packed as (shift << 32) | fo.  Flag bytes are 0, 1 (first
// occurrence) or 2 (shifted duplicate), so bit 0 and bit 1 of each byte
// count the two kinds.
constexpr int kRootVec = 4;
constexpr uint64_t kRootPerThread = 16 * kRootVec;
constexpr uint64_t kRootTile = kRootPerThread * kScanThreads;
static_assert(ROOT_FO == 1 && ROOT_SHIFT == 2, "flag bytes counted by bit");

__device__ __forceinline__ uint64_t count_word(uint32_t w) {
  return (uint64_t)__popc(w & 0x01010101u) | ((uint64_t)__popc(w & 0x02020202u) << 32);
}

// The thread's flags starting at p (p a multiple of 16); bytes at or past n
// read as ROOT_NONE.
__device__ __forceinline__ uint64_t load_flags(const uint8_t* f, uint64_t p, uint64_t n, uint4 v[kRootVec]) {
  uint64_t c = 0;
#pragma unroll
  for (int k = 0; k < kRootVec; k++) {
    const uint64_t q = p + 16 * (uint64_t)k;
    if (q + 16 <= n) {
      v[k] = *reinterpret_cast<const uint4*>(f + q);
    } else {
      uint32_t w[4] = {0, 0, 0, 0};
#pragma unroll
      for (int j = 0; j < 16; j++)
        if (q + j < n) w[j >> 2] |= (uint32_t)f[q + j] << (8 * (j & 3));
      v[k] = make_uint4(w[0], w[1], w[2], w[3]);
    }
    c += count_word(v[k].x) + count_word(v[k].y) + count_word(v[k].z) + count_word(v[k].w);
  }
  return c;
}

// The root itself is pushed only for N >= 2 in the incremental and baseline
// passes (src/tree_approach.cpp:384-393); the serial reference inserts it
// whenever it is a first occurrence (include/reference_impl.hpp:105-106).
__device__ __forceinline__ void root_prologue(const uint8_t* labels, uint32_t N, int ascending, uint32_t* fo_list,
                                              Layout* lay) {
  const uint32_t root = (labels[0] == FIRST_OCUR && (ascending || N >= 2)) ? 1u : 0u;
  lay->root_fo = root;
  if (root) fo_list[0] = 0;
}

// The first `nd` blocks issue a fused forest pass's queued inserts (only the
// assembly's ownership test and later checkpoints read them), the others
// count one tile each.
__global__ void __launch_bounds__(kScanThreads) root_count_kernel(ForestArgs a, uint32_t N, uint64_t n,
                                                                  uint64_t* tile_sums, uint32_t* fo_list,
                                                                  Layout* lay, uint32_t nd) {
  pdl_enter();
  __shared__ uint64_t sh[33];
  if (blockIdx.x < nd) {
    if (forest_fused(a)) drain_inserts(a, 0, nd);
    return;
  }
  const uint32_t tile = blockIdx.x - nd;
  if (tile == 0 && threadIdx.x == 0) root_prologue(a.labels, N, a.ascending, fo_list, lay);
  const uint64_t p = (uint64_t)tile * kRootTile + (uint64_t)threadIdx.x * kRootPerThread;
  uint4 v[kRootVec];
  const uint64_t c = p < n ? load_flags(a.rflag, p, n, v) : 0;
  uint64_t total;
  block_excl_scan(c, sh, &total);
  if (threadIdx.x == 0) tile_sums[tile] = total;
}

// Emits the roots in serial push order.  kReduce: the tile offset is the sum of
// the earlier tiles' counts (few tiles), and the last tile sets F and S;
// otherwise tile_off holds scanned offsets and root_epilogue_kernel follows.
template <bool kReduce>
__global__ void __launch_bounds__(kScanThreads) root_emit_kernel(ForestArgs a, uint64_t n, const uint64_t* tile_off,
                                                                 uint32_t* fo_list, uint32_t* sh_list, Layout* lay) {
  pdl_enter();
  __shared__ uint64_t sh[33];
  uint64_t off = 0;
  if (kReduce) {
    uint64_t part = 0;
    for (uint32_t k = threadIdx.x; k < blockIdx.x; k += blockDim.x) part += tile_off[k];
    block_excl_scan(part, sh, &off);
  } else {
    off = tile_off[blockIdx.x];
  }
  const uint64_t p = (uint64_t)blockIdx.x * kRootTile + (uint64_t)threadIdx.x * kRootPerThread;
  uint4 v[kRootVec];
  const uint64_t c = p < n ? load_flags(a.rflag, p, n, v) : 0;
  uint64_t tile_total;
  uint64_t ex = block_excl_scan(c, sh, &tile_total) + off;
  const uint32_t root = lay->root_fo;
  if (kReduce && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    lay->F = root + (uint32_t)(off + tile_total);
    lay->S = (uint32_t)((off + tile_total) >> 32);
  }
  if (!c) return;
#pragma unroll
  for (int k = 0; k < kRootVec; k++) {
    const uint32_t w4[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
      uint32_t w = w4[j];
      while (w) {
        const int bit = __ffs(w) - 1;  // lowest set flag bit: byte order = serial order
        const int byte = bit >> 3;
        const uint8_t f = (uint8_t)(w >> (8 * byte));
        const uint64_t pos = p + 16 * (uint64_t)k + 4 * j + byte;
        if (f == ROOT_FO) { fo_list[root + (uint32_t)ex] = node_at(a, pos); ex += 1; }
        else { sh_list[(uint32_t)(ex >> 32)] = node_at(a, pos); ex += 1ull << 32; }
        w &= ~(0xffu << (8 * byte));
      }
    }
  }
}

__global__ void root_epilogue_kernel(const uint64_t* total, Layout* lay) {
  pdl_enter();
  lay->F = lay->root_fo + (uint32_t)(*total);
  lay->S = (uint32_t)(*total >> 32);
}

// ---------------------------------------------------------------------------
// Diff assembly
// ---------------------------------------------------------------------------
// First-occurrence roots: region size if the root owns its digest.
__device__ __forceinline__ void fo_prep(const GatherArgs& g) {
  const uint32_t F = g.lay->F;
  const uint32_t cur = g.sp->cur;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < F; i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t node = g.fo_list[i];
    uint64_t v = 0;
    if (g.approach == APPROACH_TREE) {
      // a first-occurrence leaf owns its digest: the leaf pass demotes every
      // other one (same checkpoint id, another owner)
      bool owner = node >= g.N - 1;
      if (!owner) {
        NodeIdDev prev = slot_value(g.map, map_find(g.map, ld_digest(g.digests + node), g.err));
        owner = prev.node == node && prev.tree == cur;
      }
      if (owner) v = (1ull << 32) | num_leaf_descendents(node, g.M);
    } else {
      v = (1ull << 32) | 1ull;  // list / basic: one chunk per entry
    }
    g.fo_val[i] = v;
  }
}
struct FoEmit {
  GatherArgs g;
  __device__ __forceinline__ void operator()(uint64_t i, uint64_t ex, uint64_t v) const {
    if (!(v >> 32)) return;
    const uint32_t r = (uint32_t)(ex >> 32);
    const uint32_t node = g.fo_list[i];
    g.reg_slot[r] = (uint32_t)ex;
    g.reg_len[r] = (uint32_t)v;
    g.reg_chunk[r] = g.approach == APPROACH_TREE ? leftmost_leaf(node, g.M) - (g.N - 1) : node;
    // FO metadata: node ids (tree) or chunk ids (list, basic), 4-byte aligned
    if (g.lay->ok) *reinterpret_cast<uint32_t*>(g.stage + g.lay->pad + 32 + 4ull * r) = node;
  }
};

// Region sizes scanned with one first-occurrence root per thread (tiles of
// kFoTile) over a persistent grid: the tile count follows F on the device.
constexpr uint32_t kFoTile = kScanThreads;
__global__ void __launch_bounds__(kScanThreads) fo_tile_sums_kernel(GatherArgs g) {
  pdl_enter();
  __shared__ uint64_t sh[33];
  const uint32_t F = g.lay->F;
  const uint32_t nt = (F + kFoTile - 1) / kFoTile;
  for (uint32_t t = blockIdx.x; t < nt; t += gridDim.x) {
    const uint32_t i = t * kFoTile + threadIdx.x;
    uint64_t total;
    block_excl_scan(i < F ? g.fo_val[i] : 0, sh, &total);
    if (threadIdx.x == 0) g.scan_scratch[t] = total;
  }
}
__global__ void __launch_bounds__(kScanThreads) fo_emit_kernel(GatherArgs g) {
  pdl_enter();
  __shared__ uint64_t sh[33];
  const uint32_t F = g.lay->F;
  const uint32_t nt = (F + kFoTile - 1) / kFoTile;
  const FoEmit emit{g};
  for (uint32_t t = blockIdx.x; t < nt; t += gridDim.x) {
    const uint32_t i = t * kFoTile + threadIdx.x;
    const uint64_t v = i < F ? g.fo_val[i] : 0;
    const uint64_t ex = block_excl_scan(v, sh, nullptr) + g.scan_scratch[t];
    if (i < F) emit(i, ex, v);
  }
}

// Shifted duplicates: (source checkpoint, source node) of each root.
// The histogram of source checkpoints is warp-aggregated: most entries share
// a few keys.
__device__ __forceinline__ void shift_prep(const GatherArgs& g) {
  const uint32_t S = g.lay->S;
  const uint32_t cur = g.sp->cur;
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x; b < S; b += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = b + threadIdx.x;
    uint32_t key = 0xffffffffu;
    if (i < S) {
      uint32_t node = g.sh_list[i];
      int64_t slot = map_find(g.map, ld_digest(g.digests + node), g.err);
      NodeIdDev prev = slot_value(g.map, slot);
      if (slot < 0 || prev.tree > cur) { atomicOr(g.err, DERR_MISSING); prev.tree = 0; prev.node = 0; }
      g.sh_key[i] = prev.tree;
      g.sh_prev[i] = prev.node;
      key = prev.tree;
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    if (key != 0xffffffffu && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&g.hist[key], (uint32_t)__popc(peers));
  }
}

// Both root lists' lookups in one launch.
__global__ void roots_prep_kernel(GatherArgs g) {
  pdl_enter();
  shift_prep(g);
  fo_prep(g);
}

// One block: repeat-count table, layout, header; bin representatives for the
// list approach's BinOp1D.
// First, the tile sums of the region-size scan become tile offsets in place,
// and their total gives the region count and the data chunk count.
__global__ void layout_kernel(GatherArgs g) {
  pdl_enter();
  __shared__ uint64_t sh[33];
  Layout* lay = g.lay;
  {
    const uint32_t ntiles = (lay->F + kFoTile - 1) / kFoTile;
    uint64_t carry = 0;
    for (uint32_t b = 0; b < ntiles; b += blockDim.x) {
      const uint32_t i = b + threadIdx.x;
      const uint64_t v = i < ntiles ? g.scan_scratch[i] : 0;
      uint64_t t;
      const uint64_t ex = block_excl_scan(v, sh, &t);
      if (i < ntiles) g.scan_scratch[i] = carry + ex;
      carry += t;
    }
    if (threadIdx.x == 0) {
      lay->num_distinct = (uint32_t)(carry >> 32);
      lay->chunk_counter = (uint32_t)carry;
    }
    __syncthreads();
  }
  const uint32_t cur = g.sp->cur;
  const uint32_t K = cur + 1;
  const uint32_t F = lay->F, S = lay->S, nd = lay->num_distinct;
  // P = number of source checkpoints that occur; max_key = largest of them
  __shared__ uint32_t smax;
  if (threadIdx.x == 0) {
    smax = 0;
    lay->nkeys = 0;  // set below once the keys are known
    lay->sort_n = 0;
    lay->sort_tiles = 0;
  }
  __syncthreads();
  uint32_t P = 0;
  for (uint32_t b = 0; b < K; b += blockDim.x) {
    uint32_t k = b + threadIdx.x;
    uint64_t nz = (k < K && g.hist[k] > 0) ? 1 : 0;
    uint64_t t;
    block_excl_scan(nz, sh, &t);
    P += (uint32_t)t;
    if (nz) atomicMax(&smax, k);
  }
  __syncthreads();
  const uint32_t max_key = smax;
  const uint64_t fo_off = 32;
  const uint64_t meta_meta = g.approach == APPROACH_BASIC ? 0 : 1;
  const uint64_t data_off = fo_off + 4ull * F + meta_meta * (8ull * P + 8ull * S);
  const uint64_t pad = (16 - (data_off & 15)) & 15;
  const uint64_t data_len_bytes = (uint64_t)lay->chunk_counter * g.cs;
  uint64_t diff_len = data_off + data_len_bytes;
  if (threadIdx.x == 0) {
    lay->P = meta_meta ? P : 0;
    lay->pad = pad;
    lay->data_off = data_off;
    lay->table_off = fo_off + 4ull * nd;
    lay->pairs_off = fo_off + 4ull * nd + 8ull * P;
    if (pad + diff_len > g.stage_cap) {
      atomicOr(g.err, DERR_CAPACITY);
      lay->diff_len = 0;
      lay->ok = 0;
    } else {
      lay->diff_len = diff_len;
      lay->ok = 1;
    }
    // datasizes as the reference's collect_diff returns them
    if (g.approach == APPROACH_TREE) {
      uint64_t meta = 4ull * F + 8ull * P + 8ull * S;
      lay->size_data = diff_len - meta;  // src/tree_approach.cpp:707-709
      lay->size_meta = meta;
    } else if (g.approach == APPROACH_LIST) {
      uint64_t dsz = (uint64_t)g.cs * F;  // src/list_approach.cpp:241-246
      lay->size_data = dsz;
      lay->size_meta = diff_len - dsz;
    } else {
      uint32_t dsz = F * g.cs;  // src/basic_approach.cpp:141-142 (32-bit product)
      lay->size_data = dsz;
      lay->size_meta = diff_len - dsz;
    }
  }
  __syncthreads();
  if (!lay->ok) return;
  uint8_t* diff = g.stage + pad;
  if (threadIdx.x == 0) {
    // header_t, include/utils.hpp:29-37
    uint32_t* h32 = reinterpret_cast<uint32_t*>(diff);
    h32[0] = g.sp->baseline_id;
    h32[1] = cur;
    h32[2] = (uint32_t)g.len;
    h32[3] = (uint32_t)(g.len >> 32);
    h32[4] = g.cs;
    h32[5] = F;
    h32[6] = meta_meta ? P : 0;
    h32[7] = meta_meta ? S : 0;
  }
  if (!meta_meta) return;
  // zero bytes that the reference leaves at zero when F != num_distinct
  for (uint64_t b = 32 + 4ull * nd + 8ull * P + 8ull * S + threadIdx.x; b < data_off; b += blockDim.x) diff[b] = 0;
  // (checkpoint id, count) table in ascending id (src/tree_approach.cpp:657-665)
  uint32_t base = 0;
  for (uint32_t b = 0; b < K; b += blockDim.x) {
    uint32_t k = b + threadIdx.x;
    uint64_t nz = (k < K && g.hist[k] > 0) ? 1 : 0;
    uint64_t t;
    uint64_t ex = block_excl_scan(nz, sh, &t);
    if (nz) {
      uint32_t* e = reinterpret_cast<uint32_t*>(diff + lay->table_off + 8ull * (base + ex));
      e[0] = k;
      e[1] = g.hist[k];
    }
    base += (uint32_t)t;
  }
  // sort representative of each key: stable sort by BinOp1D bin equals stable
  // sort by the smallest key sharing the bin
  const uint32_t nbins = g.approach == APPROACH_TREE ? cur : S;
  const double range = (double)(g.approach == APPROACH_TREE ? cur : max_key);
  const double mul = (range <= (double)nbins) ? 1.0 : (double)nbins / range;
  for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) {
    int bk = (int)(mul * (double)k);
    uint32_t rep = k;
    while (rep > 0 && (int)(mul * (double)(rep - 1)) == bk) rep--;
    g.rep[k] = rep;
    g.rank[k] = 0;
  }
  __syncthreads();
  // dense index of each representative that some present key maps to
  for (uint32_t k = threadIdx.x; k < K; k += blockDim.x)
    if (g.hist[k] > 0) g.rank[g.rep[k]] = 1;
  __syncthreads();
  uint32_t run = 0;
  for (uint32_t b0 = 0; b0 < K; b0 += blockDim.x) {
    uint32_t k = b0 + threadIdx.x;
    uint64_t v = k < K ? g.rank[k] : 0;
    uint64_t t;
    uint64_t ex = block_excl_scan(v, sh, &t);
    if (k < K) g.rank[k] = run + (uint32_t)ex;
    run += (uint32_t)t;
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < K; k += blockDim.x)
    if (g.hist[k] > 0) g.rep[k] = g.rank[g.rep[k]];
  if (threadIdx.x == 0) {
    lay->nkeys = run;
    const uint32_t T = (S + kSortTile - 1) / kSortTile;
    lay->sort_tiles = T;
    lay->sort_n = run * T;
    if (run > kSortFastKeys) atomicOr(g.err, DERR_SORTKEYS);
  }
}

// Stable counting sort of the shift entries by representative key.
// Tile t counts its keys; matrix[key * T + t] (key-major).
__global__ void sort_count_kernel(GatherArgs g) {
  pdl_enter();
  extern __shared__ uint32_t cnt[];
  const uint32_t K = g.lay->nkeys, S = g.lay->S, T = g.lay->sort_tiles;
  if (K > kSortFastKeys) return;
  for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) {
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    const uint64_t b = (uint64_t)t * kSortTile;
    // every load of the tile issued before the first count
    constexpr int kPer = kSortTile / 256;
    uint32_t key[kPer];
#pragma unroll
    for (int j = 0; j < kPer; j++) {
      const uint64_t i = b + threadIdx.x + 256ull * j;
      key[j] = i < S ? g.sh_key[i] : 0xffffffffu;
    }
#pragma unroll
    for (int j = 0; j < kPer; j++) key[j] = key[j] != 0xffffffffu ? g.rep[key[j]] : 0xffffffffu;
#pragma unroll
    for (int j = 0; j < kPer; j++)
      if (key[j] != 0xffffffffu) atomicAdd(&cnt[key[j]], 1u);
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) g.sort_mat[(uint64_t)k * T + t] = cnt[k];
    __syncthreads();
  }
}
struct MatVal {
  const uint64_t* m;
  __device__ __forceinline__ uint64_t operator()(uint64_t i) const { return m[i]; }
};
struct MatEmit {
  uint64_t* m;
  __device__ __forceinline__ void operator()(uint64_t i, uint64_t ex, uint64_t) const { m[i] = ex; }
};
// Stable placement of the shift entries of one 4096-entry tile: 8 warps each
// rank a contiguous 512-entry slice in order (per-warp key counters in shared
// memory), then the per-key counts of earlier warps and the tile's global
// base (key-major scan of sort_mat) give each entry its position.
constexpr int kSortWarps = 8;
__global__ void __launch_bounds__(256) sort_scatter_kernel(GatherArgs g) {
  pdl_enter();
  __shared__ uint32_t keys[kSortTile];
  __shared__ uint32_t lrank[kSortTile];
  extern __shared__ uint32_t cnt[];  // [kSortWarps][K]
  const uint32_t K = g.lay->nkeys, S = g.lay->S, T = g.lay->sort_tiles;
  if (!g.lay->ok || K > kSortFastKeys) return;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr uint32_t kSlice = kSortTile / kSortWarps;
  uint8_t* pairs = g.stage + g.lay->pad + g.lay->pairs_off;
  for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) {
    const uint64_t b = (uint64_t)t * kSortTile;
    if (b >= S) break;
    const uint32_t n = (uint32_t)(S - b < kSortTile ? S - b : kSortTile);
    constexpr int kPer = kSortTile / 256;
    {
      uint32_t kk[kPer];
#pragma unroll
      for (int j = 0; j < kPer; j++) {
        const uint32_t i = threadIdx.x + 256u * j;
        kk[j] = i < n ? g.sh_key[b + i] : 0;
      }
#pragma unroll
      for (int j = 0; j < kPer; j++) {
        const uint32_t i = threadIdx.x + 256u * j;
        if (i < n) keys[i] = g.rep[kk[j]];
      }
    }
    for (uint32_t k = threadIdx.x; k < kSortWarps * K; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    uint32_t* wc = cnt + warp * K;
    for (uint32_t i0 = warp * kSlice; i0 < (warp + 1) * kSlice && i0 < n; i0 += 32) {
      const uint32_t i = i0 + lane;
      const bool v = i < n && i < (warp + 1) * kSlice;
      const uint32_t key = v ? keys[i] : 0xffffffffu;
      const uint32_t peers = __match_any_sync(0xffffffffu, key);
      const uint32_t rank = __popc(peers & ((1u << lane) - 1));
      uint32_t base = v ? wc[key] : 0;
      __syncwarp();
      if (v) {
        lrank[i] = base + rank;
        if (lane == (uint32_t)(__ffs(peers) - 1)) wc[key] = base + __popc(peers);
      }
      __syncwarp();
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) {
      uint32_t run = (uint32_t)g.sort_mat[(uint64_t)k * T + t];
      for (int w = 0; w < kSortWarps; w++) {
        uint32_t c = cnt[w * K + k];
        cnt[w * K + k] = run;
        run += c;
      }
    }
    __syncthreads();
    {
      uint32_t nd[kPer], pv[kPer];
#pragma unroll
      for (int j = 0; j < kPer; j++) {
        const uint32_t i = threadIdx.x + 256u * j;
        nd[j] = i < n ? g.sh_list[b + i] : 0;
        pv[j] = i < n ? g.sh_prev[b + i] : 0;
      }
#pragma unroll
      for (int j = 0; j < kPer; j++) {
        const uint32_t i = threadIdx.x + 256u * j;
        if (i >= n) continue;
        const uint32_t pos = cnt[(i / kSlice) * K + keys[i]] + lrank[i];
        uint32_t* e = reinterpret_cast<uint32_t*>(pairs + 8ull * pos);  // 4-byte aligned only
        e[0] = nd[j];
        e[1] = pv[j];
      }
    }
    __syncthreads();
  }
}

// Chunk gather into the data section.  Regions (reg_chunk, reg_slot, reg_len)
// are sorted by slot; every 16-byte unit of the data section is written once.
// Each block owns a contiguous range of units, so a thread locates its region
// once by binary search and then walks forward.
__global__ void copy_kernel(GatherArgs g) {
  pdl_enter();
  if (!g.lay->ok) return;
  const uint32_t R = g.lay->num_distinct;
  const uint64_t nslots = g.lay->chunk_counter;
  if (R == 0 || nslots == 0) return;
  uint8_t* dst = g.stage + g.lay->pad + g.lay->data_off;
  const uint64_t cs = g.cs;
  const uint64_t last = (uint64_t)g.N - 1;
  const uint64_t tail_len = g.len - last * cs;  // bytes of the last chunk
  const uint64_t nunits = nslots * cs / 16;
  const uint64_t per_block = ((nunits + gridDim.x - 1) / gridDim.x + blockDim.x - 1) / blockDim.x * blockDim.x;
  const uint64_t u0 = (uint64_t)blockIdx.x * per_block, u1 = min(u0 + per_block, nunits);
  uint64_t u = u0 + threadIdx.x;
  if (u >= u1) return;
  // 16-byte units per chunk; a power of two (every usual chunk size) is a shift
  const uint64_t upc = cs / 16;
  const int lg = (upc & (upc - 1)) == 0 ? __ffsll((long long)upc) - 1 : -1;
  auto slot_of_unit = [&](uint64_t uu) { return lg >= 0 ? uu >> lg : uu / upc; };
  uint64_t slot = slot_of_unit(u);
  uint32_t lo = 0, hi = R - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (g.reg_slot[mid] <= slot) lo = mid; else hi = mid - 1;
  }
  uint32_t r = lo;
  // one 16-byte unit of the data section; chunks past the end of the buffer
  // stay zero (the reference reads out of bounds there)
  auto load = [&](uint64_t uu) {
    const uint64_t sl = slot_of_unit(uu);
    while (r + 1 < R && g.reg_slot[r + 1] <= sl) r++;
    const uint64_t within = (uu - sl * upc) * 16;
    const uint64_t chunk = (uint64_t)g.reg_chunk[r] + (sl - g.reg_slot[r]);
    uint4 v = make_uint4(0, 0, 0, 0);
    if (chunk < last || (chunk == last && within + 16 <= tail_len)) {
      v = __ldcs(reinterpret_cast<const uint4*>(g.data + chunk * cs + within));
    } else if (chunk == last && within < tail_len) {
      uint32_t w[4] = {0, 0, 0, 0};
      for (uint32_t b = 0; b < 16 && within + b < tail_len; b++) w[b >> 2] |= (uint32_t)g.data[chunk * cs + within + b] << (8 * (b & 3));
      v = make_uint4(w[0], w[1], w[2], w[3]);
    }
    return v;
  };
  // two units in flight per thread: both loads issue before either store
  for (; u < u1; u += 2 * (uint64_t)blockDim.x) {
    const uint64_t ub = u + blockDim.x;
    const uint4 va = load(u);
    const uint4 vb = ub < u1 ? load(ub) : make_uint4(0, 0, 0, 0);
    __stcs(reinterpret_cast<uint4*>(dst + u * 16), va);
    if (ub < u1) __stcs(reinterpret_cast<uint4*>(dst + ub * 16), vb);
  }
}

// Byte-granular gather for chunk sizes that are not multiples of 16 or
// buffers that are not 16-byte aligned.
__global__ void copy_bytes_kernel(GatherArgs g) {
  pdl_enter();
  if (!g.lay->ok) return;
  const uint32_t R = g.lay->num_distinct;
  const uint64_t nslots = g.lay->chunk_counter;
  if (R == 0 || nslots == 0) return;
  uint8_t* dst = g.stage + g.lay->pad + g.lay->data_off;
  const uint64_t cs = g.cs;
  const uint64_t nbytes = nslots * cs;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nbytes; b += stride) {
    uint64_t slot = b / cs;
    uint32_t lo = 0, hi = R - 1;
    while (lo < hi) {
      uint32_t mid = (lo + hi + 1) >> 1;
      if (g.reg_slot[mid] <= slot) lo = mid; else hi = mid - 1;
    }
    const uint64_t chunk = (uint64_t)g.reg_chunk[lo] + (slot - g.reg_slot[lo]);
    const uint64_t src = chunk * cs + (b - slot * cs);
    dst[b] = src < g.len ? g.data[src] : 0;
  }
}

// list / basic: flags over chunks -> ascending FO (changed) and SHIFT lists
struct ChunkVal {
  const uint8_t* labels;
  int basic;
  __device__ __forceinline__ uint64_t operator()(uint64_t c) const {
    uint8_t l = labels[c];
    if (basic) return l ? 1ull : 0ull;
    return (l == FIRST_OCUR ? 1ull : 0ull) | (l == SHIFT_DUPL ? (1ull << 32) : 0ull);
  }
};
struct ChunkEmit {
  uint32_t* fo_list;
  uint32_t* sh_list;
  __device__ __forceinline__ void operator()(uint64_t c, uint64_t ex, uint64_t v) const {
    if (v & 1ull) fo_list[(uint32_t)ex] = (uint32_t)c;
    if (v >> 32) sh_list[(uint32_t)(ex >> 32)] = (uint32_t)c;
  }
};
__global__ void chunk_totals_kernel(const uint64_t* total, Layout* lay) {
  pdl_enter();
  lay->root_fo = 0;
  lay->F = (uint32_t)(*total);
  lay->S = (uint32_t)(*total >> 32);
}

// Entries of a table moved into a larger one (keys are stored already
// mapped, and unique, so every claim is new).
__global__ void map_rehash_kernel(DigestMap from, uint64_t from_cap, DigestMap to, uint32_t* err) {
  uint32_t created = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < from_cap; i += (uint64_t)gridDim.x * blockDim.x) {
    const MapSlot& s = from.slots[i];
    const uint4 v = *reinterpret_cast<const uint4*>(s.key);
    if (key_empty(v)) continue;
    uint64_t slot;
    if (map_claim(to, Digest{{v.x, v.y, v.z, v.w}}, &slot, err) != INS_NEW) continue;
    to.slots[slot].win = s.win;
    to.slots[slot].tree = s.tree;
    created++;
  }
  count_new_entries(to, created);
}

// Epochs of every entry set to 0, before the engine's epoch counter restarts.
__global__ void map_rebase_kernel(DigestMap m, uint64_t cap) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (uint64_t)gridDim.x * blockDim.x) {
    MapSlot& s = m.slots[i];
    if (s.win != kWinEmpty) s.win &= (1ull << kPrioBits) - 1;
  }
}

}  // namespace

cudaError_t launch_map_rehash(const DigestMap& from, uint64_t from_cap, const DigestMap& to, uint32_t* err,
                              cudaStream_t s) {
  map_rehash_kernel<<<grid_for(from_cap, 256), 256, 0, s>>>(from, from_cap, to, err);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_map_rebase(const DigestMap& m, uint64_t cap, cudaStream_t s) {
  map_rebase_kernel<<<grid_for(cap, 256), 256, 0, s>>>(m, cap);
  note_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
cudaError_t launch_forest(const ForestArgs& a, int pass, int baseline, uint32_t N, cudaStream_t s) {
  if (N < 2) return cudaSuccess;
  if (pass == 0) {
    // the duplicate pass (alone or fused into the first) writes only the
    // flags of roots; every other position (node 1 .. M-1 in canonical
    // order) reads ROOT_NONE
    cudaError_t e = cudaMemsetAsync(a.rflag, ROOT_NONE, 2ull * N - 2, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.ins_count, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
  }
  // deepest interior depth: that of node N-2
  uint32_t dmax = 0;
  while (((2ull << dmax) - 1) <= (uint64_t)(N - 2)) dmax++;
  const bool dup_baseline = pass == 1 && baseline;
  int bot = (int)dmax;
  if (!dup_baseline && dmax + 1 >= kBottomLevels) {
    const uint32_t top = dmax - (kBottomLevels - 1);
    const uint64_t first = (1ull << top) - 1;
    const uint64_t count = std::min<uint64_t>(1ull << top, (uint64_t)N - 1 - first);
    if (a.hash_kind == HASH_MD5) launch_k(forest_bottom12_kernel<HASH_MD5>, (uint32_t)count, 256, 0, s, a, pass, N, top);
    else launch_k(forest_bottom12_kernel<HASH_MURMUR3>, (uint32_t)count, 256, 0, s, a, pass, N, top);
    note_launch();
    bot = (int)top - 1;
  }
  for (; bot >= 0; bot -= kSpanLevels) {
    const uint32_t top = bot >= (int)kSpanLevels - 1 ? (uint32_t)bot - (kSpanLevels - 1) : 0;
    const uint64_t first = (1ull << top) - 1;
    const uint64_t count = std::min<uint64_t>(1ull << top, (uint64_t)N - 1 - first);
    if (!dup_baseline && (uint32_t)bot - top == kSpanLevels - 1)
      if (a.hash_kind == HASH_MD5) launch_k(forest_span9_warp_kernel<HASH_MD5>, (uint32_t)count, 256, 0, s, a, pass, N, top);
      else launch_k(forest_span9_warp_kernel<HASH_MURMUR3>, (uint32_t)count, 256, 0, s, a, pass, N, top);
    else
      launch_k(forest_span_kernel, (uint32_t)count, 256, 0, s, a, pass, baseline, N, top, (uint32_t)bot);
    note_launch();
    if (top == 0) break;
  }
  if (pass == 0) {
    launch_k(forest_insert_kernel, grid_for(N, 256), 256, 0, s, a);
    note_launch();
  }
  return cudaGetLastError();
}

cudaError_t launch_root_compaction(const ForestArgs& fa, uint32_t N, uint32_t M, uint32_t* fo_list,
                                   uint32_t* sh_list, Layout* lay, uint64_t* scan_scratch, uint64_t* scan_total,
                                   cudaStream_t s) {
  const uint64_t n = (uint64_t)M - 1;  // every node but the root
  uint32_t ntiles = (uint32_t)((n + kRootTile - 1) / kRootTile);
  if (ntiles == 0) ntiles = 1;
  const uint32_t nd = 2 * num_sms();
  launch_k(root_count_kernel, ntiles + nd, kScanThreads, 0, s, fa, N, n, scan_scratch, fo_list, lay, nd);
  if (ntiles <= reduce_tile_limit()) {
    launch_k(root_emit_kernel<true>, ntiles, kScanThreads, 0, s, fa, n, scan_scratch, fo_list, sh_list, lay);
    note_launch(2);
    return cudaGetLastError();
  }
  launch_k(scan_tile_offsets_kernel, 1, 1024, 0, s, scan_scratch, ntiles, scan_total);
  launch_k(root_emit_kernel<false>, ntiles, kScanThreads, 0, s, fa, n, scan_scratch, fo_list, sh_list, lay);
  launch_k(root_epilogue_kernel, 1, 1, 0, s, scan_total, lay);
  note_launch(4);
  return cudaGetLastError();
}

cudaError_t launch_chunk_compaction(const uint8_t* labels, uint32_t n_chunks, int basic, uint32_t* fo_list,
                                    uint32_t* sh_list, Layout* lay, uint64_t* scan_scratch, uint64_t* scan_total,
                                    cudaStream_t s) {
  cudaError_t e = grid_scan(ChunkVal{labels, basic}, ChunkEmit{fo_list, sh_list}, nullptr, n_chunks, scan_scratch,
                            scan_total, s);
  if (e != cudaSuccess) return e;
  launch_k(chunk_totals_kernel, 1, 1, 0, s, scan_total, lay);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_assemble(const GatherArgs& g, uint64_t max_entries, cudaStream_t s) {
  cudaError_t e;
  // the FO metadata is written while scanning, so the pad must be known first:
  // pad depends on F, P, S; P needs the histogram.  Order: shift prep
  // (histogram), FO prep + scan (region sizes), layout (pad, table, header),
  // FO emit (metadata + regions), sort, copy.
  cudaMemsetAsync(g.hist, 0, sizeof(uint32_t) * (size_t)g.k_cap, s);
  const uint32_t gs = grid_for(max_entries, 256);
  launch_k(roots_prep_kernel, gs, 256, 0, s, g);
  // region totals first (phase 1+2 of the scan), then layout, then emit
  const uint32_t gfo = (uint32_t)std::min<uint64_t>((max_entries + kFoTile - 1) / kFoTile + 1, 4ull * num_sms());
  launch_k(fo_tile_sums_kernel, gfo, kScanThreads, 0, s, g);
  launch_k(layout_kernel, 1, 1024, 0, s, g);
  launch_k(fo_emit_kernel, gfo, kScanThreads, 0, s, g);
  note_launch(4);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (g.approach != APPROACH_BASIC) {
    // bound on the distinct keys (source checkpoints): at most k_cap, which
    // covers every checkpoint id that this launch sequence can see
    const uint32_t K = std::min<uint32_t>(g.k_cap, kSortFastKeys);
    const uint32_t T = (uint32_t)((max_entries + kSortTile - 1) / kSortTile) + 1;
    const size_t smem_cnt = sizeof(uint32_t) * (size_t)K;
    const size_t smem_sc = sizeof(uint32_t) * (size_t)K * kSortWarps;
    static size_t attr_sc = 0;
    if (smem_sc > 16 * 1024 && smem_sc > attr_sc) {
      cudaFuncSetAttribute(sort_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_sc);
      attr_sc = smem_sc;
    }
    // tiles of the actual shift entries, read on the device: small grids
    const uint32_t gsort = std::min<uint32_t>(T, 2 * num_sms());
    launch_k(sort_count_kernel, gsort, 256, smem_cnt, s, g);
    e = grid_scan(MatVal{g.sort_mat}, MatEmit{g.sort_mat}, &g.lay->sort_n, (uint64_t)K * T, g.scan_scratch2,
                  g.scan_total2, s);
    if (e != cudaSuccess) return e;
    launch_k(sort_scatter_kernel, gsort, 256, smem_sc, s, g);
    note_launch(2);
  }
  const bool vec = (g.cs % 16 == 0) && ((reinterpret_cast<uintptr_t>(g.data) & 15) == 0);
  static const bool reg = (register_input_kernel(reinterpret_cast<const void*>(copy_kernel), INPUT_GATHER),
                           register_input_kernel(reinterpret_cast<const void*>(copy_bytes_kernel), INPUT_GATHER), true);
  (void)reg;
  if (vec) launch_k(copy_kernel, num_sms() * 8, 256, 0, s, g);
  else launch_k(copy_bytes_kernel, num_sms() * 8, 256, 0, s, g);
  note_launch();
  return cudaGetLastError();
}

}  // namespace mtc
