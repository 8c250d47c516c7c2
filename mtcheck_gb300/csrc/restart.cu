// restart.cu -- rebuilding a checkpoint from its chain of incremental
// checkpoints (TreeDeduplicator::restart_chkpt, src/tree_approach.cpp:713-1128;
// ListDeduplicator::restart_chkpt, src/list_approach.cpp:259-574;
// BasicDeduplicator::restart_chkpt, src/basic_approach.cpp:155-321).
//
// The reference walks the chain one checkpoint at a time and, at every step,
// visits every chunk whose provenance (node_list) points at that checkpoint.
// Here the walk is reorganised for the GPU without changing its result:
//   1. the metadata of every checkpoint of the chain is decoded in bulk;
//   2. the main checkpoint's scatter is resolved per chunk with last-writer
//      ranks (its regions are copied in serial order, later ones win);
//   3. for every later step the keys it covers are written into per-step
//      first-insert-wins tables plus a per-key bitmask of covering steps;
//   4. every chunk then follows its own provenance down the chain: a chunk
//      that a step does not cover only moves to the next step, so it jumps
//      straight to the next step whose mask bit is set;
//   5. one gather pass copies each chunk once from the diff that owns it.
// A chunk that the reference never writes is not written here either.
#include <algorithm>
#include <cstring>

#include "engine.hpp"
#include "mtc_scan.cuh"

namespace mtc {

namespace {

constexpr uint64_t kNone = ~0ull;
constexpr uint32_t kOffBits = 48;

struct DiffInfo {
  const uint8_t* base;
  uint64_t len;
  uint64_t fo_off, cnt_off, map_off, data_off;
  uint32_t F, P, S, id;
  uint32_t fo_begin, sh_begin, rrs_begin, pad;
};

struct RArgs {
  int approach;
  uint32_t N, M, cs;
  uint64_t datalen;
  uint32_t ndiff, nsteps, W, K;  // K keys per step table
  uint32_t cur_main;             // id of the main checkpoint
  const DiffInfo* di;
  uint32_t nfo, nsh;
  uint32_t *fo_node, *fo_seg, *fo_clen;
  uint64_t* fo_excl;
  uint32_t *sh_node, *sh_prev, *sh_tree, *sh_seg;
  uint64_t *sh_off, *sh_excl;
  uint32_t* rrs;
  uint64_t *nl, *res, *nl_rank, *cp_rank;
  uint32_t* fo_at;  // main checkpoint: lowest FO entry per node (tree) or chunk (list)
  uint32_t *dm_tab, *rm_tab, *dm_mask, *rm_mask;
  uint64_t *dm_excl, *rm_excl;  // per-entry item prefix of the chain tables
  uint4* fo_rng;                // chain FO entries: leaf key ranges {lo0, n0, lo1, n1}
  uint2 *bnd0, *bnd1;           // per expansion tile: first and last entry
  uint32_t max_tiles;           // capacity of bnd0 / bnd1
  uint64_t *tot;                // [0] dm items, [1] rm items, [2] main FO chunks, [3] main shift chunks
  uint8_t* out;
  uint32_t* err;
};

__device__ __forceinline__ uint32_t rd32(const uint8_t* p) {
  // diff sections are 4-byte aligned relative to the header
  uint32_t v;
  memcpy(&v, p, 4);
  return v;
}

__device__ __forceinline__ uint32_t seg_of(const DiffInfo* di, uint32_t ndiff, uint32_t g, bool fo) {
  uint32_t lo = 0, hi = ndiff - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if ((fo ? di[mid].fo_begin : di[mid].sh_begin) <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// 1. decode FO and shift entries of every diff
__global__ void load_entries_kernel(RArgs a) {
  const uint64_t total = (uint64_t)a.nfo + a.nsh;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (uint64_t)gridDim.x * blockDim.x) {
    if (g < a.nfo) {
      uint32_t s = seg_of(a.di, a.ndiff, (uint32_t)g, true);
      const DiffInfo& d = a.di[s];
      uint32_t i = (uint32_t)g - d.fo_begin;
      uint32_t node = rd32(d.base + d.fo_off + 4ull * i);
      if (a.approach == APPROACH_TREE ? node > a.M : node >= a.N) { atomicOr(a.err, DERR_RANGE); node = 0; }
      a.fo_node[g] = node;
      a.fo_seg[g] = s;
    } else {
      uint32_t h = (uint32_t)(g - a.nfo);
      uint32_t s = seg_of(a.di, a.ndiff, h, false);
      const DiffInfo& d = a.di[s];
      uint32_t i = h - d.sh_begin;
      uint32_t node = rd32(d.base + d.map_off + 8ull * i), prev = rd32(d.base + d.map_off + 8ull * i + 4);
      if (a.approach == APPROACH_TREE ? (node > a.M || prev > a.M) : node >= a.N) {
        atomicOr(a.err, DERR_RANGE);
        node = 0;
        prev = 0;
      }
      a.sh_node[h] = node;
      a.sh_prev[h] = prev;
      a.sh_seg[h] = s;
    }
  }
}

// 2. inclusive prefix of the repeat-count table of every diff over ids 0..id
//    (src/tree_approach.cpp:868-883); a table naming an id above the diff's
//    own id is corrupt
__global__ void rrs_kernel(RArgs a) {
  for (uint32_t s = blockIdx.x; s < a.ndiff; s += gridDim.x) {
    const DiffInfo& d = a.di[s];
    uint32_t* r = a.rrs + d.rrs_begin;
    for (uint32_t j = threadIdx.x; j <= d.id; j += blockDim.x) r[j] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (uint32_t i = 0; i < d.P; i++) {
        uint32_t ck = rd32(d.base + d.cnt_off + 8ull * i);
        uint32_t n = rd32(d.base + d.cnt_off + 8ull * i + 4);
        if (ck > d.id) { atomicOr(a.err, DERR_RANGE); continue; }
        r[ck] = n;
      }
      uint32_t acc = 0;
      for (uint32_t j = 0; j <= d.id; j++) { acc += r[j]; r[j] = acc; }
    }
    __syncthreads();
  }
}

// 3. source checkpoint of every shift entry: the smallest j with i < prefix[j]
//    (src/tree_approach.cpp:894-898), 0 if none
__global__ void shift_tree_kernel(RArgs a) {
  for (uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; h < a.nsh; h += (uint64_t)gridDim.x * blockDim.x) {
    const DiffInfo& d = a.di[a.sh_seg[h]];
    const uint32_t i = (uint32_t)h - d.sh_begin;
    const uint32_t* r = a.rrs + d.rrs_begin;
    uint32_t lo = 0, hi = d.id + 1;  // first j in [0, id] with r[j] > i
    while (lo < hi) {
      uint32_t mid = (lo + hi) >> 1;
      if (r[mid] > i) hi = mid; else lo = mid + 1;
    }
    a.sh_tree[h] = lo <= d.id ? lo : 0;
  }
}

// region length of an FO entry (tree: num_leaf_descendents, list/basic: 1)
struct FoLen {
  const uint32_t* node;
  uint32_t M;
  int tree;
  __device__ __forceinline__ uint64_t operator()(uint64_t g) const { return tree ? num_leaf_descendents(node[g], M) : 1; }
};
struct StoreExcl {
  uint64_t* out;
  __device__ __forceinline__ void operator()(uint64_t g, uint64_t ex, uint64_t) const { out[g] = ex; }
};
// chunk_len of each FO entry relative to its own diff (src/tree_approach.cpp:803-816)
__global__ void clen_kernel(RArgs a) {
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < a.nfo; g += (uint64_t)gridDim.x * blockDim.x) {
    const DiffInfo& d = a.di[a.fo_seg[g]];
    a.fo_clen[g] = (uint32_t)(a.fo_excl[g] - a.fo_excl[d.fo_begin]);
  }
}

// main checkpoint (segment 0): lowest FO entry per node / chunk
__global__ void fo_at_kernel(RArgs a) {
  const uint32_t F = a.di[0].F;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < F; i += (uint64_t)gridDim.x * blockDim.x)
    atomicMin(&a.fo_at[a.fo_node[i]], (uint32_t)i);  // node range checked while decoding
}

// distinct_map lookup of (node, cur) in the main checkpoint's tree: the FO
// entry with the smallest index whose inserted node set contains `node`
// (src/tree_approach.cpp:825-848 inserts the root and every level below it
// while the level's first node is < num_nodes, clipping the last level at
// num_nodes).  Returns the byte offset or kNone.
__device__ uint64_t main_dm_lookup(const RArgs& a, uint32_t node) {
  if (node > a.M) return kNone;
  uint32_t best = 0xffffffffu;
  uint32_t u = node;
  uint64_t scale = 1;  // 2^k: relative depth of `node` below u
  while (true) {
    uint32_t i = a.fo_at[u];
    if (i != 0xffffffffu && i < best) {
      bool in = true;
      if (scale > 1) {
        // node is a proper descendant; its level is visited only if the
        // level's first node is below num_nodes
        uint64_t left = scale * ((uint64_t)u + 1) - 1;
        in = left < a.M;
      }
      if (in) best = i;
    }
    if (u == 0) break;
    u = (u - 1) >> 1;
    scale <<= 1;
  }
  if (best == 0xffffffffu) return kNone;
  const uint32_t start = leftmost_leaf(a.fo_node[best], a.M);
  const uint32_t leaf = leftmost_leaf(node, a.M);
  return (uint64_t)(uint32_t)(a.fo_clen[best] + leaf - start) * a.cs;
}

// main shift entries: copy source offset (src/tree_approach.cpp:887-903,
// src/list_approach.cpp:376-394)
__global__ void main_shift_kernel(RArgs a) {
  const DiffInfo& d = a.di[0];
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < d.S; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t prev = a.sh_prev[i], tree = a.sh_tree[i];
    uint64_t off = 0;
    if (tree == d.id) {
      if (a.approach == APPROACH_TREE) {
        uint64_t v = main_dm_lookup(a, prev);
        if (v != kNone) off = v;
      } else if (prev < a.N && a.fo_at[prev] != 0xffffffffu) {
        off = (uint64_t)a.fo_at[prev] * a.cs;
      }
    }
    a.sh_off[i] = off;
  }
}
// chunks touched by a main shift entry (tree: num_leaf_descendents(prev))
struct MainShiftLen {
  const uint32_t* prev;
  uint32_t M;
  int tree;
  __device__ __forceinline__ uint64_t operator()(uint64_t i) const { return tree ? num_leaf_descendents(prev[i], M) : 1; }
};

__device__ __forceinline__ uint32_t upper_entry(const uint64_t* excl, uint32_t n, uint64_t item) {
  // last entry e with excl[e] <= item
  uint32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (excl[mid] <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Items numbered by an exclusive prefix over entries are processed in tiles of
// kExpandTile per block: the entries overlapping a tile (each entry has at
// least one item) are staged in shared memory once, and every item finds its
// entry by a binary search there instead of in global memory.
constexpr uint32_t kExpandTile = 2048;
struct ExpandTile {
  uint64_t ex[kExpandTile + 1];
  uint32_t e0, cnt;
};
// The first and last entry of every tile, for all tiles at once, written
// from the entries' side: entry k owns items [excl[k], excl[k+1]) and records
// itself for every tile that starts or ends inside that range.  No dependent
// loads (a per-tile binary search would chain ~log2(n) of them).
__global__ void expand_bounds_kernel(const uint64_t* excl, uint32_t n, const uint64_t* total, uint2* bounds,
                                     uint32_t max_tiles) {
  const uint64_t tot = *total;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = excl[k], e = k + 1 < n ? excl[k + 1] : tot;
    if (e <= s) continue;  // no items: never the owner of one
    for (uint64_t b = s / kExpandTile; b * kExpandTile < e && b < max_tiles; b++) {
      const uint64_t first = b * kExpandTile;
      const uint64_t last = (first + kExpandTile < tot ? first + kExpandTile : tot) - 1;
      if (first >= s) bounds[b].x = (uint32_t)k;
      if (last >= s && last < e) bounds[b].y = (uint32_t)k;
    }
  }
}

__device__ __forceinline__ void expand_stage(ExpandTile& T, const uint64_t* excl, uint32_t n, uint64_t t0,
                                             uint64_t t1, const uint2* bounds = nullptr,
                                             uint32_t max_tiles = 0) {
  if (threadIdx.x == 0) {
    const uint64_t b = t0 / kExpandTile;  // tiles start at multiples of kExpandTile
    uint32_t e0, e1;
    if (bounds && b < max_tiles) {
      const uint2 v = bounds[b];
      e0 = v.x;
      e1 = v.y;
    } else {
      e0 = upper_entry(excl, n, t0);
      e1 = upper_entry(excl, n, t1 - 1);
    }
    T.e0 = e0;
    T.cnt = e1 - e0 + 1;
  }
  __syncthreads();
  const uint32_t cnt = T.cnt <= kExpandTile + 1 ? T.cnt : 0;
  for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) T.ex[i] = excl[T.e0 + i];
  __syncthreads();
}
__device__ __forceinline__ uint32_t expand_entry(const ExpandTile& T, const uint64_t* excl, uint32_t n,
                                                 uint64_t item) {
  if (T.cnt > kExpandTile + 1) return upper_entry(excl, n, item);
  uint32_t lo = 0, hi = T.cnt - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (T.ex[mid] <= item) lo = mid; else hi = mid - 1;
  }
  return T.e0 + lo;
}

// main scatter: which entry writes node_list / copies each chunk last
// (src/tree_approach.cpp:825-925; ranks: FO entries 1+i, shift entries 2^32+i)
// which = 0: FO regions (prefix fo_excl, total tot[2]); 1: shift regions
// (prefix sh_excl, total tot[3])
__global__ void __launch_bounds__(256) main_cover_kernel(RArgs a, int which) {
  __shared__ ExpandTile T;
  const DiffInfo& d = a.di[0];
  const uint64_t total = a.tot[2 + which];
  const uint64_t* excl = which ? a.sh_excl : a.fo_excl;
  const uint32_t n = which ? d.S : d.F;
  const bool tree = a.approach == APPROACH_TREE;
  for (uint64_t t0 = (uint64_t)blockIdx.x * kExpandTile; t0 < total; t0 += (uint64_t)gridDim.x * kExpandTile) {
    const uint64_t t1 = t0 + kExpandTile < total ? t0 + kExpandTile : total;
    expand_stage(T, excl, n, t0, t1, which ? a.bnd1 : a.bnd0, a.max_tiles);
    for (uint64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
      const uint32_t i = expand_entry(T, excl, n, t);
      const uint32_t j = (uint32_t)(t - excl[i]);
      if (which == 0) {
        uint64_t c = tree ? (uint64_t)(uint32_t)(leftmost_leaf(a.fo_node[i], a.M) - (a.N - 1) + j) : a.fo_node[i];
        if (c >= a.N) continue;
        const unsigned long long r = 1ull + i;
        atomicMax(reinterpret_cast<unsigned long long*>(&a.nl_rank[c]), r);
        atomicMax(reinterpret_cast<unsigned long long*>(&a.cp_rank[c]), r);
      } else {
        uint64_t c = tree ? (uint64_t)(uint32_t)(leftmost_leaf(a.sh_node[i], a.M) - (a.N - 1) + j) : a.sh_node[i];
        if (c >= a.N) continue;
        const unsigned long long r = (1ull << 32) + i;
        atomicMax(reinterpret_cast<unsigned long long*>(&a.nl_rank[c]), r);
        if (a.sh_tree[i] == d.id) atomicMax(reinterpret_cast<unsigned long long*>(&a.cp_rank[c]), r);
      }
    }
    __syncthreads();
  }
}

__device__ __forceinline__ uint64_t pack_nl(uint32_t node, uint32_t tree) { return ((uint64_t)tree << 32) | node; }

// node_list and first copy source of every chunk after the main checkpoint
__global__ void main_resolve_kernel(RArgs a) {
  const DiffInfo& d = a.di[0];
  const uint32_t cur = d.id;
  const bool tree = a.approach == APPROACH_TREE;
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.N; c += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t nr = a.nl_rank[c], cr = a.cp_rank[c];
    uint64_t nl;
    if (nr == 0) {
      // "same as previous" (src/tree_approach.cpp:932-937)
      nl = pack_nl(tree ? (uint32_t)c + a.N - 1 : (uint32_t)c, cur - 1);
    } else if (nr < (1ull << 32)) {
      nl = pack_nl((uint32_t)c, cur);
    } else {
      const uint32_t i = (uint32_t)(nr - (1ull << 32));
      if (tree) {
        const uint32_t j = (uint32_t)c - (leftmost_leaf(a.sh_node[i], a.M) - (a.N - 1));
        nl = pack_nl(leftmost_leaf(a.sh_prev[i], a.M) + j, a.sh_tree[i]);
      } else {
        nl = pack_nl(a.sh_prev[i], a.sh_tree[i]);
      }
    }
    a.nl[c] = nl;
    uint64_t res = kNone;
    if (cr != 0) {
      if (cr < (1ull << 32)) {
        const uint32_t i = (uint32_t)(cr - 1);
        uint64_t base = tree ? (uint64_t)a.fo_clen[i] * a.cs : (uint64_t)i * a.cs;
        uint64_t within = tree ? (c - (leftmost_leaf(a.fo_node[i], a.M) - (a.N - 1))) * (uint64_t)a.cs : 0;
        res = base + within;
      } else {
        const uint32_t i = (uint32_t)(cr - (1ull << 32));
        uint64_t within = tree ? (c - (leftmost_leaf(a.sh_node[i], a.M) - (a.N - 1))) * (uint64_t)a.cs : 0;
        res = a.sh_off[i] + within;
      }
      if (res >= (1ull << kOffBits)) res = kNone;
    }
    a.res[c] = res;
  }
}

// ---------------------------------------------------------------------------
// chain tables
// ---------------------------------------------------------------------------
// leaves of the node set that distinct_map holds for a tree FO entry rooted at u
// (u itself, or its descendants at the levels the insertion loop visits),
// as at most two ranges of node ids within [N-1, M].
__device__ __forceinline__ int fo_leaf_ranges(uint32_t u, uint32_t N, uint32_t M, uint32_t lo[2], uint32_t hi[2]) {
  int n = 0;
  if (u >= N - 1) {
    if (u <= M) { lo[0] = u; hi[0] = u; n = 1; }
    return n;
  }
  uint64_t scale = 2;
  while (true) {
    uint64_t left = scale * ((uint64_t)u + 1) - 1;
    if (left >= M) break;
    uint64_t right = left + scale - 1;
    uint64_t a = left > (uint64_t)(N - 1) ? left : (uint64_t)(N - 1);
    uint64_t b = right < (uint64_t)M ? right : (uint64_t)M;
    if (a <= b && n < 2) { lo[n] = (uint32_t)a; hi[n] = (uint32_t)b; n++; }
    scale <<= 1;
  }
  return n;
}

// Per chain FO entry, once: the (at most two) leaf ranges its distinct map
// covers, or for the list and basic approaches its one chunk.
__global__ void chain_ranges_kernel(RArgs a, uint32_t n) {
  const bool tree = a.approach == APPROACH_TREE;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t g = a.di[1].fo_begin + k;  // chain entries follow the main ones
    uint4 r = make_uint4(0, 0, 0, 0);
    if (tree) {
      uint32_t lo[2], hi[2];
      const int nr = fo_leaf_ranges(a.fo_node[g], a.N, a.M, lo, hi);
      if (nr > 0) { r.x = lo[0]; r.y = hi[0] - lo[0] + 1; }
      if (nr > 1) { r.z = lo[1]; r.w = hi[1] - lo[1] + 1; }
    } else {
      r.x = a.fo_node[g];
      r.y = 1;
    }
    a.fo_rng[g] = r;
  }
}

struct ChainDmCount {
  RArgs a;
  __device__ __forceinline__ uint64_t operator()(uint64_t k) const {
    const uint4 r = a.fo_rng[a.di[1].fo_begin + k];
    return (uint64_t)r.y + r.w;
  }
};
struct ChainRmCount {
  RArgs a;
  __device__ __forceinline__ uint64_t operator()(uint64_t k) const {
    const uint64_t h = a.di[1].sh_begin + k;
    if (a.approach == APPROACH_LIST) return 1;
    const uint32_t node = a.sh_node[h];
    // repeat_map keys: the root (src/tree_approach.cpp:1069) and the leaf
    // range of num_leaf_descendents(node) from leftmost_leaf(node) (:1073-1078);
    // only keys in [N-1, M] can be looked up by a leaf
    uint64_t c = num_leaf_descendents(node, a.M);
    if (node >= a.N - 1 && node <= a.M) c += 1;
    return c;
  }
};

__device__ __forceinline__ uint32_t key_of_leaf(const RArgs& a, uint32_t x) { return x - (a.N - 1); }

// pass 0: set the initial value of every covered table cell and its mask bit;
// pass 1: lowest rank wins.  which = 0: distinct-map keys of the FO entries,
// 1: repeat-map keys of the shift entries.
__global__ void __launch_bounds__(256) chain_tables_kernel(RArgs a, int pass, int which) {
  __shared__ ExpandTile T;
  if (a.nsteps == 0) return;
  const uint64_t total = a.tot[which];
  const uint32_t n = which ? a.nsh - a.di[1].sh_begin : a.nfo - a.di[1].fo_begin;
  const uint64_t* excl = which ? a.rm_excl : a.dm_excl;
  const bool tree = a.approach == APPROACH_TREE;
  for (uint64_t t0 = (uint64_t)blockIdx.x * kExpandTile; t0 < total; t0 += (uint64_t)gridDim.x * kExpandTile) {
    const uint64_t t1 = t0 + kExpandTile < total ? t0 + kExpandTile : total;
    expand_stage(T, excl, n, t0, t1, which ? a.bnd1 : a.bnd0, a.max_tiles);
    for (uint64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
      const uint32_t k = expand_entry(T, excl, n, t);
      uint64_t j = t - excl[k];
      uint32_t key, rank, s;
      if (which == 0) {
        const uint64_t g = a.di[1].fo_begin + k;  // chain entries follow the main ones
        s = a.fo_seg[g] - 1;
        rank = (uint32_t)g - a.di[1 + s].fo_begin;
        const uint4 r = a.fo_rng[g];
        if (tree) {
          const uint32_t x = j < r.y ? r.x + (uint32_t)j : r.z + (uint32_t)(j - r.y);
          key = key_of_leaf(a, x);
        } else {
          key = r.x;
          if (key >= a.N) continue;
        }
      } else {
        const uint64_t h = a.di[1].sh_begin + k;
        s = a.sh_seg[h] - 1;
        const uint32_t i = (uint32_t)h - a.di[1 + s].sh_begin;
        if (tree) {
          const uint32_t node = a.sh_node[h];
          const uint32_t len = num_leaf_descendents(node, a.M);
          if (j < len) {
            const uint32_t x = leftmost_leaf(node, a.M) + (uint32_t)j;
            if (x < a.N - 1 || x > a.M) continue;
            key = key_of_leaf(a, x);
            rank = 2 * i + 1;
          } else {
            key = key_of_leaf(a, node);
            rank = 2 * i;
          }
        } else {
          key = a.sh_node[h];
          if (key >= a.N) continue;
          rank = 2 * i;
        }
      }
      uint32_t* tab = (which ? a.rm_tab : a.dm_tab) + (uint64_t)s * a.K + key;
      if (pass == 0) {
        *tab = 0xffffffffu;
        atomicOr((which ? a.rm_mask : a.dm_mask) + (uint64_t)key * a.W + (s >> 5), 1u << (s & 31));
      } else {
        atomicMin(tab, rank);
      }
    }
    __syncthreads();
  }
}

// offset of leaf/chunk x in step s's data through its distinct map, or kNone
__device__ __forceinline__ uint64_t chain_dm_offset(const RArgs& a, uint32_t s, uint32_t x) {
  const bool tree = a.approach == APPROACH_TREE;
  uint32_t key;
  if (tree) {
    if (x < a.N - 1 || x > a.M) return kNone;
    key = key_of_leaf(a, x);
  } else {
    if (x >= a.N) return kNone;
    key = x;
  }
  if (!(a.dm_mask[(uint64_t)key * a.W + (s >> 5)] & (1u << (s & 31)))) return kNone;
  const uint32_t i = a.dm_tab[(uint64_t)s * a.K + key];
  if (!tree) return (uint64_t)i * a.cs;
  const uint64_t g = a.di[1 + s].fo_begin + i;
  return (uint64_t)(uint32_t)(a.fo_clen[g] + x - leftmost_leaf(a.fo_node[g], a.M)) * a.cs;
}

// 4. per-chunk walk down the chain (src/tree_approach.cpp:1083-1118,
//    src/list_approach.cpp:520-567, src/basic_approach.cpp:293-312)
__global__ void walk_kernel(RArgs a) {
  if (a.nsteps == 0) return;
  const uint32_t id0 = a.cur_main - 1;              // id of step 0
  const uint32_t idl = id0 - (a.nsteps - 1);       // id of the last step
  const bool tree = a.approach == APPROACH_TREE;
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.N; c += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t nl = a.nl[c];
    uint32_t x = (uint32_t)nl, t = (uint32_t)(nl >> 32);
    for (uint32_t hop = 0; hop <= a.nsteps + 1; hop++) {
      if (t > id0 || t < idl) break;  // owned by the main checkpoint, or beyond the chain
      uint32_t key;
      if (tree) {
        if (x < a.N - 1 || x > a.M) { atomicOr(a.err, DERR_INTERIOR); break; }
        key = key_of_leaf(a, x);
      } else {
        if (x >= a.N) break;
        key = x;
      }
      // next step at or below t that mentions this key
      uint32_t s = id0 - t, found = 0xffffffffu;
      for (uint32_t w = s >> 5; w < a.W; w++) {
        uint32_t m = a.dm_mask[(uint64_t)key * a.W + w] | a.rm_mask[(uint64_t)key * a.W + w];
        if (w == (s >> 5)) m &= ~0u << (s & 31);
        if (m) { found = w * 32 + __ffs(m) - 1; break; }
      }
      if (found >= a.nsteps) break;  // never mentioned again: left as is
      s = found;
      const uint32_t ts = id0 - s;
      const uint64_t off = chain_dm_offset(a, s, x);
      if (off != kNone) {
        if (off < (1ull << kOffBits)) a.res[c] = ((uint64_t)(1 + s) << kOffBits) | off;
        break;
      }
      if (a.approach == APPROACH_BASIC) break;
      const uint32_t r = a.rm_tab[(uint64_t)s * a.K + key];
      const uint64_t h = a.di[1 + s].sh_begin + (r >> 1);
      uint32_t pnode, ptree = a.sh_tree[h];
      if (tree && (r & 1)) pnode = leftmost_leaf(a.sh_prev[h], a.M) + (x - leftmost_leaf(a.sh_node[h], a.M));
      else pnode = a.sh_prev[h];
      if (ptree == ts) {
        const uint64_t o2 = chain_dm_offset(a, s, pnode);
        if (o2 != kNone && o2 < (1ull << kOffBits)) a.res[c] = ((uint64_t)(1 + s) << kOffBits) | o2;
        break;
      }
      x = pnode;
      t = ptree;
    }
  }
}

// 5. one copy per chunk from the diff that owns it; one thread per 16-byte
//    unit of the output, two units in flight (chunk sizes that are not
//    multiples of 16 go byte by byte)
struct GatherUnit {
  const uint8_t* src;
  uint8_t* dst;
  uint32_t n;  // bytes to copy, 0 for none
};
__device__ __forceinline__ GatherUnit gather_unit(const RArgs& a, uint64_t u, uint64_t upc, int lg) {
  GatherUnit g{nullptr, nullptr, 0};
  const uint64_t cs = a.cs;
  const uint64_t c = lg >= 0 ? u >> lg : u / upc;
  const uint64_t byte = u * 16, within = (u - c * upc) * 16;
  const uint64_t r = a.res[c];
  if (r == kNone) return g;
  const DiffInfo& d = a.di[r >> kOffBits];
  const uint64_t off = d.data_off + (r & ((1ull << kOffBits) - 1)) + within;
  uint64_t n = 16;
  if (byte + n > a.datalen) n = a.datalen - byte;
  if (c * cs + cs > a.datalen && within + n > a.datalen - c * cs) n = a.datalen - c * cs - within;
  if (off >= d.len) return g;
  if (off + n > d.len) n = d.len - off;
  g.src = d.base + off;
  g.dst = a.out + byte;
  g.n = (uint32_t)n;
  return g;
}
__device__ __forceinline__ void gather_copy(const GatherUnit& g, const uint4& v) {
  if (g.n == 16 && (((uintptr_t)g.src | (uintptr_t)g.dst) & 15) == 0) {
    *reinterpret_cast<uint4*>(g.dst) = v;
  } else if (g.n == 16 && (((uintptr_t)g.src | (uintptr_t)g.dst) & 3) == 0) {
    const uint32_t* s4 = reinterpret_cast<const uint32_t*>(g.src);
    *reinterpret_cast<uint4*>(g.dst) = make_uint4(s4[0], s4[1], s4[2], s4[3]);
  } else {
    for (uint32_t b = 0; b < g.n; b++) g.dst[b] = g.src[b];
  }
}
__device__ __forceinline__ uint4 gather_load(const GatherUnit& g) {
  if (g.n == 16 && (((uintptr_t)g.src | (uintptr_t)g.dst) & 15) == 0)
    return __ldcs(reinterpret_cast<const uint4*>(g.src));
  return make_uint4(0, 0, 0, 0);
}
__global__ void gather_kernel(RArgs a) {
  const uint64_t cs = a.cs;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  if (cs % 16 == 0) {
    const uint64_t units = (a.datalen + 15) / 16;
    const uint64_t upc = cs / 16;  // units per chunk; a power of two is a shift
    const int lg = (upc & (upc - 1)) == 0 ? __ffsll((long long)upc) - 1 : -1;
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < units; u += 2 * stride) {
      const GatherUnit g0 = gather_unit(a, u, upc, lg);
      const GatherUnit g1 = u + stride < units ? gather_unit(a, u + stride, upc, lg) : GatherUnit{nullptr, nullptr, 0};
      const uint4 v0 = gather_load(g0), v1 = gather_load(g1);
      if (g0.n) gather_copy(g0, v0);
      if (g1.n) gather_copy(g1, v1);
    }
    return;
  }
  for (uint64_t byte = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; byte < a.datalen; byte += stride) {
    const uint64_t c = byte / cs, within = byte - c * cs;
    const uint64_t r = a.res[c];
    if (r == kNone) continue;
    const DiffInfo& d = a.di[r >> kOffBits];
    const uint64_t off = d.data_off + (r & ((1ull << kOffBits) - 1)) + within;
    if (off < d.len) a.out[byte] = d.base[off];
  }
}

inline uint32_t gsz(uint64_t n, int threads = 256, int per_sm = 8) {
  uint64_t g = (n + threads - 1) / threads;
  uint64_t cap = (uint64_t)num_sms() * per_sm;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return (uint32_t)g;
}

}  // namespace

// Restart scratch owned by the engine between calls.
struct RestartScratch {
  DevBuf<DiffInfo> di;
  DevBuf<uint32_t> fo_node, fo_seg, fo_clen, sh_node, sh_prev, sh_tree, sh_seg, rrs, fo_at, dm_tab, rm_tab, dm_mask,
      rm_mask;
  DevBuf<uint64_t> fo_excl, sh_off, sh_excl, nl, res, nl_rank, cp_rank, dm_excl, rm_excl, tot, scan, scan_total;
  DevBuf<uint4> fo_rng;
  DevBuf<uint2> bnd0, bnd1;
};

void destroy_restart_scratch(RestartScratch* r) { delete r; }

static void set_scratch_pool(RestartScratch* r, cudaMemPool_t pool) {
  r->di.pool = pool;
  r->fo_rng.pool = pool;
  r->bnd0.pool = pool;
  r->bnd1.pool = pool;
  for (auto* b : {&r->fo_node, &r->fo_seg, &r->fo_clen, &r->sh_node, &r->sh_prev, &r->sh_tree, &r->sh_seg, &r->rrs,
                  &r->fo_at, &r->dm_tab, &r->rm_tab, &r->dm_mask, &r->rm_mask})
    b->pool = pool;
  for (auto* b : {&r->fo_excl, &r->sh_off, &r->sh_excl, &r->nl, &r->res, &r->nl_rank, &r->cp_rank, &r->dm_excl,
                  &r->rm_excl, &r->tot, &r->scan, &r->scan_total})
    b->pool = pool;
}

int Engine::restart(uint8_t* dev_out, uint64_t len, const std::vector<const uint8_t*>& dev_diffs,
                    const std::vector<uint64_t>& lens, const std::vector<HeaderHost>& headers, uint32_t id) {
  if (int rc = order_inputs()) return rc;
  int rc = restart_enqueue(dev_out, len, dev_diffs, lens, headers, id);
  if (rc) return rc;
  MTC_CUDA_R(cudaStreamSynchronize(stream_));
  return restart_complete();
}

int Engine::restart_complete() {
  float ms = 0;
  cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
  restart_timers[1] = ms * 1e-3;
  if (restart_raw_) return ST_OK;
  const uint32_t herr = err_host_[0];
  last_device_error = herr;
  if (herr & DERR_RANGE) return fail(ST_ECORRUPT, "restart metadata out of range");
  if (herr & DERR_INTERIOR) return fail(ST_ENOTSUP, "restart provenance names an interior node");
  return ST_OK;
}

int Engine::restart_enqueue(uint8_t* dev_out, uint64_t len, const std::vector<const uint8_t*>& dev_diffs,
                            const std::vector<uint64_t>& lens, const std::vector<HeaderHost>& headers, uint32_t id) {
  cudaStream_t s = stream_;
  if (id >= dev_diffs.size()) return fail(ST_EINVAL, "checkpoint id outside the chain");
  if (spilled_) return fail(ST_EINVAL, "state spilled to host: restore it first");
  cudaEvent_t e0 = ev_[0], e1 = ev_[1];
  cudaEventRecord(e0, s);
  restart_raw_ = mode_ == MODE_FULL;
  if (mode_ == MODE_FULL) {
    // FullDeduplicator::restart copies the raw checkpoint (src/full_approach.cpp:122-141)
    if (lens[id] != len) return fail(ST_EINVAL, "output length differs from the checkpoint");
    MTC_CUDA_R(cudaMemcpyAsync(dev_out, dev_diffs[id], len, cudaMemcpyDeviceToDevice, s));
    cudaEventRecord(e1, s);
    return ST_OK;
  }
  const int approach = mode_ == MODE_LIST ? APPROACH_LIST : mode_ == MODE_BASIC ? APPROACH_BASIC : APPROACH_TREE;
  const bool basic = approach == APPROACH_BASIC;
  const HeaderHost& H = headers[id];
  if (lens[id] < sizeof(HeaderHost)) return fail(ST_ECORRUPT, "checkpoint shorter than its header");
  if (H.chunk_size == 0) return fail(ST_ECORRUPT, "chunk size 0 in header");
  if (H.datalen != len) return fail(ST_EINVAL, "output length differs from header.datalen");
  const uint64_t n64 = (H.datalen + H.chunk_size - 1) / H.chunk_size;
  if (n64 == 0 || n64 >= (1ull << 31)) return fail(ST_ENOTSUP, "chunk count out of range");
  const uint32_t N = (uint32_t)n64, M = 2 * N - 1, cs = H.chunk_size;

  // chain steps exactly as the reference's loop visits them
  // (src/tree_approach.cpp:943, src/list_approach.cpp:428, src/basic_approach.cpp:247)
  std::vector<uint32_t> steps;
  {
    int64_t ref = H.ref_id;
    for (int64_t idx = (int64_t)id - 1; idx >= ref && idx >= 0; idx--) {
      steps.push_back((uint32_t)idx);
      ref = headers[idx].ref_id;
    }
  }
  const uint32_t nsteps = (uint32_t)steps.size();
  std::vector<uint32_t> slots(1, id);
  for (uint32_t x : steps) slots.push_back(x);
  std::vector<DiffInfo> di(slots.size());
  uint32_t nfo = 0, nsh = 0, nrrs = 0;
  for (size_t k = 0; k < slots.size(); k++) {
    const uint32_t idx = slots[k];
    const HeaderHost& h = headers[idx];
    if (lens[idx] < sizeof(HeaderHost)) return fail(ST_ECORRUPT, "checkpoint shorter than its header");
    if (h.chunk_size != cs || h.datalen != H.datalen)
      return fail(ST_ENOTSUP, "chain mixes chunk sizes or buffer lengths");
    if (k > 0 && h.chkpt_id != H.chkpt_id - (uint32_t)k)
      return fail(ST_ENOTSUP, "chain checkpoint ids are not consecutive");
    if (h.chkpt_id > (1u << 24)) return fail(ST_ENOTSUP, "checkpoint id too large");
    DiffInfo& d = di[k];
    d.base = dev_diffs[idx];
    d.len = lens[idx];
    d.F = h.num_first_ocur;
    d.P = basic ? 0 : h.num_prior_chkpts;
    d.S = basic ? 0 : h.num_shift_dupl;
    d.id = h.chkpt_id;
    d.fo_off = 32;
    d.cnt_off = 32 + 4ull * d.F;
    d.map_off = d.cnt_off + 8ull * d.P;
    d.data_off = d.map_off + 8ull * d.S;
    if (d.data_off > d.len) return fail(ST_ECORRUPT, "metadata runs past the end of a checkpoint");
    d.fo_begin = nfo;
    d.sh_begin = nsh;
    d.rrs_begin = nrrs;
    nfo += d.F;
    nsh += d.S;
    nrrs += d.id + 1;
  }
  const uint32_t W = (nsteps + 31) / 32 ? (nsteps + 31) / 32 : 1;
  const uint32_t K = approach == APPROACH_TREE ? N + 1 : N;
  if (!rs_) {
    rs_ = new RestartScratch();
    if (pool_) set_scratch_pool(rs_, pool_);
  }
  RestartScratch& R = *rs_;
  MTC_CUDA_R(R.di.ensure(di.size(), s));
  MTC_CUDA_R(cudaMemcpyAsync(R.di.p, di.data(), sizeof(DiffInfo) * di.size(), cudaMemcpyHostToDevice, s));
  MTC_CUDA_R(R.fo_node.ensure(nfo + 1, s));
  MTC_CUDA_R(R.fo_seg.ensure(nfo + 1, s));
  MTC_CUDA_R(R.fo_rng.ensure(nfo + 1, s));
  // expansion tiles: a chain step covers at most every leaf of its tree twice
  const uint64_t max_items = (uint64_t)(nsteps + 2) * 2ull * M + nfo + nsh + 16;
  const uint32_t max_tiles = (uint32_t)std::min<uint64_t>(max_items / kExpandTile + 2, 1u << 26);
  MTC_CUDA_R(R.bnd0.ensure(max_tiles, s));
  MTC_CUDA_R(R.bnd1.ensure(max_tiles, s));
  MTC_CUDA_R(R.fo_clen.ensure(nfo + 1, s));
  MTC_CUDA_R(R.fo_excl.ensure(nfo + 1, s));
  MTC_CUDA_R(R.sh_node.ensure(nsh + 1, s));
  MTC_CUDA_R(R.sh_prev.ensure(nsh + 1, s));
  MTC_CUDA_R(R.sh_tree.ensure(nsh + 1, s));
  MTC_CUDA_R(R.sh_seg.ensure(nsh + 1, s));
  MTC_CUDA_R(R.sh_off.ensure(nsh + 1, s));
  MTC_CUDA_R(R.sh_excl.ensure(nsh + 1, s));
  MTC_CUDA_R(R.rrs.ensure(nrrs + 1, s));
  MTC_CUDA_R(R.nl.ensure(N, s));
  MTC_CUDA_R(R.res.ensure(N, s));
  MTC_CUDA_R(R.nl_rank.ensure(N, s));
  MTC_CUDA_R(R.cp_rank.ensure(N, s));
  MTC_CUDA_R(R.fo_at.ensure((size_t)M + 2, s));
  MTC_CUDA_R(R.dm_excl.ensure(nfo + 1, s));
  MTC_CUDA_R(R.rm_excl.ensure(nsh + 1, s));
  MTC_CUDA_R(R.tot.ensure(4, s));
  MTC_CUDA_R(R.dm_tab.ensure((size_t)std::max<uint32_t>(nsteps, 1) * K, s));
  MTC_CUDA_R(R.rm_tab.ensure((size_t)std::max<uint32_t>(nsteps, 1) * K, s));
  MTC_CUDA_R(R.dm_mask.ensure((size_t)K * W, s));
  MTC_CUDA_R(R.rm_mask.ensure((size_t)K * W, s));
  const uint64_t scan_n = std::max<uint64_t>(nfo, nsh) + 1;
  MTC_CUDA_R(R.scan.ensure(scan_n / kScanTile + 2, s));
  MTC_CUDA_R(R.scan_total.ensure(1, s));
  MTC_CUDA_R(err_.ensure(1, s));
  MTC_CUDA_R(cudaMemsetAsync(err_.p, 0, sizeof(uint32_t), s));

  RArgs a{};
  a.approach = approach;
  a.N = N; a.M = M; a.cs = cs; a.datalen = H.datalen;
  a.ndiff = (uint32_t)di.size(); a.nsteps = nsteps; a.W = W; a.K = K; a.cur_main = H.chkpt_id;
  a.di = R.di.p;
  a.nfo = nfo; a.nsh = nsh;
  a.fo_node = R.fo_node.p; a.fo_seg = R.fo_seg.p; a.fo_clen = R.fo_clen.p; a.fo_excl = R.fo_excl.p;
  a.sh_node = R.sh_node.p; a.sh_prev = R.sh_prev.p; a.sh_tree = R.sh_tree.p; a.sh_seg = R.sh_seg.p;
  a.sh_off = R.sh_off.p; a.sh_excl = R.sh_excl.p;
  a.rrs = R.rrs.p;
  a.nl = R.nl.p; a.res = R.res.p; a.nl_rank = R.nl_rank.p; a.cp_rank = R.cp_rank.p;
  a.fo_at = R.fo_at.p;
  a.dm_tab = R.dm_tab.p; a.rm_tab = R.rm_tab.p; a.dm_mask = R.dm_mask.p; a.rm_mask = R.rm_mask.p;
  a.dm_excl = R.dm_excl.p; a.rm_excl = R.rm_excl.p; a.tot = R.tot.p;
  a.fo_rng = R.fo_rng.p;
  a.bnd0 = R.bnd0.p;
  a.bnd1 = R.bnd1.p;
  a.max_tiles = max_tiles;
  a.out = dev_out; a.err = err_.p;
  const bool tree = approach == APPROACH_TREE;

  // 1-3: decode entries, repeat tables, source checkpoints
  if (nfo + nsh) { load_entries_kernel<<<gsz((uint64_t)nfo + nsh), 256, 0, s>>>(a); note_launch(); }
  rrs_kernel<<<gsz(di.size(), 1, 4), 256, 0, s>>>(a);
  note_launch();
  if (nsh) { shift_tree_kernel<<<gsz(nsh), 256, 0, s>>>(a); note_launch(); }
  // chunk_len of every FO entry within its own diff
  if (nfo) {
    MTC_CUDA_R(grid_scan(FoLen{R.fo_node.p, M, tree ? 1 : 0}, StoreExcl{R.fo_excl.p}, nullptr, nfo, R.scan.p,
                         R.scan_total.p, s));
    clen_kernel<<<gsz(nfo), 256, 0, s>>>(a);
    note_launch();
  }
  // main checkpoint
  MTC_CUDA_R(cudaMemsetAsync(R.fo_at.p, 0xff, sizeof(uint32_t) * ((size_t)M + 2), s));
  MTC_CUDA_R(cudaMemsetAsync(R.nl_rank.p, 0, sizeof(uint64_t) * N, s));
  MTC_CUDA_R(cudaMemsetAsync(R.cp_rank.p, 0, sizeof(uint64_t) * N, s));
  if (di[0].F) { fo_at_kernel<<<gsz(di[0].F), 256, 0, s>>>(a); note_launch(); }
  if (di[0].S) { main_shift_kernel<<<gsz(di[0].S), 256, 0, s>>>(a); note_launch(); }
  // items of the main scatter: FO regions (prefix = chunk_len), shift regions
  MTC_CUDA_R(cudaMemsetAsync(R.tot.p, 0, sizeof(uint64_t) * 4, s));
  if (di[0].F) {
    MTC_CUDA_R(grid_scan(FoLen{R.fo_node.p, M, tree ? 1 : 0}, StoreExcl{R.fo_excl.p}, nullptr, di[0].F, R.scan.p,
                         R.tot.p + 2, s));
  }
  if (di[0].S) {
    MTC_CUDA_R(grid_scan(MainShiftLen{R.sh_prev.p, M, tree ? 1 : 0}, StoreExcl{R.sh_excl.p}, nullptr, di[0].S,
                         R.scan.p, R.tot.p + 3, s));
  }
  if (di[0].F) {
    expand_bounds_kernel<<<num_sms() * 2, 256, 0, s>>>(R.fo_excl.p, di[0].F, R.tot.p + 2, R.bnd0.p, a.max_tiles);
    note_launch();
  }
  if (di[0].S) {
    expand_bounds_kernel<<<num_sms() * 2, 256, 0, s>>>(R.sh_excl.p, di[0].S, R.tot.p + 3, R.bnd1.p, a.max_tiles);
    note_launch();
  }
  main_cover_kernel<<<num_sms() * 4, 256, 0, s>>>(a, 0);
  main_cover_kernel<<<num_sms() * 4, 256, 0, s>>>(a, 1);
  main_resolve_kernel<<<gsz(N), 256, 0, s>>>(a);
  note_launch(3);
  // chain
  if (nsteps) {
    MTC_CUDA_R(cudaMemsetAsync(R.dm_mask.p, 0, sizeof(uint32_t) * (size_t)K * W, s));
    MTC_CUDA_R(cudaMemsetAsync(R.rm_mask.p, 0, sizeof(uint32_t) * (size_t)K * W, s));
    const uint32_t nfo_chain = nfo - di[1].fo_begin, nsh_chain = nsh - di[1].sh_begin;
    if (nfo_chain) {
      chain_ranges_kernel<<<gsz(nfo_chain), 256, 0, s>>>(a, nfo_chain);
      note_launch();
    }
    if (nfo_chain)
      MTC_CUDA_R(grid_scan(ChainDmCount{a}, StoreExcl{R.dm_excl.p}, nullptr, nfo_chain, R.scan.p, R.tot.p + 0, s));
    if (nsh_chain && !basic)
      MTC_CUDA_R(grid_scan(ChainRmCount{a}, StoreExcl{R.rm_excl.p}, nullptr, nsh_chain, R.scan.p, R.tot.p + 1, s));
    if (nfo_chain) {
      expand_bounds_kernel<<<num_sms() * 2, 256, 0, s>>>(R.dm_excl.p, nfo_chain, R.tot.p + 0, R.bnd0.p,
                                                         a.max_tiles);
      note_launch();
    }
    if (nsh_chain && !basic) {
      expand_bounds_kernel<<<num_sms() * 2, 256, 0, s>>>(R.rm_excl.p, nsh_chain, R.tot.p + 1, R.bnd1.p,
                                                         a.max_tiles);
      note_launch();
    }
    // per table: every cell initialised (pass 0) before the lowest rank wins (pass 1)
    for (int which = 0; which < 2; which++)
      for (int pass = 0; pass < 2; pass++)
        chain_tables_kernel<<<num_sms() * 4, 256, 0, s>>>(a, pass, which);
    walk_kernel<<<gsz(N), 256, 0, s>>>(a);
    note_launch(5);
  }
  gather_kernel<<<num_sms() * 16, 256, 0, s>>>(a);
  note_launch();
  cudaEventRecord(e1, s);
  MTC_CUDA_R(cudaMemcpyAsync(err_host_, err_.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  return ST_OK;
}

}  // namespace mtc
