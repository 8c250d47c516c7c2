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
//      first-insert-wins tables plus a per-key bitmask of covering steps
//      (one launch; cells carry a per-restart epoch, so the tables are
//      never cleared);
//   4. every chunk then follows its own provenance down the chain: a chunk
//      that a step does not cover only moves to the next step, so it jumps
//      straight to the next step whose mask bit is set; the result is the
//      chunk's source address and byte count;
//   5. one copy pass moves each chunk once from the diff that owns it.
// A chunk that the reference never writes is not written here either.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "engine.hpp"
#include "mtc_scan.cuh"

namespace mtc {

namespace {

constexpr uint64_t kNone = ~0ull;
// a resolved data offset at or above 2^kOffBits (only a corrupt chain gives
// one) leaves the chunk as it was, like an offset past the diff's end
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
  uint32_t F0, S0;               // FO and shift entries of the main checkpoint
  uint32_t fo_cb, sh_cb;         // first FO / shift entry of the chain (nfo / nsh without one)
  uint64_t tag;                  // this restart's epoch << 32 (chain table cells)
  uint32_t *fo_node, *fo_seg, *fo_clen;
  uint64_t* fo_excl;
  uint32_t *sh_node, *sh_prev, *sh_tree, *sh_seg;
  uint64_t *sh_off, *sh_excl;
  uint32_t* rrs;
  uint64_t *nl_rank, *cp_rank;  // main scatter ranks, tagged: ntag | rank (older tags read as 0)
  uint64_t ntag;                 // this restart's epoch << 34
  uint64_t* srcp;                // per chunk: source address (TMA restore path)
  uint32_t* nbv;                 // per chunk: bytes to copy, 0 for none
  uint32_t* fo_at;  // main checkpoint: lowest FO entry per node (tree) or chunk (list)
  uint32_t* dm_off;              // [step][key] position of the key's chunk in the step's data (valid
                                 // where the step's distinct-map bit is set)
  uint64_t* rm_tab;              // [step][key] repeat-map cells, tag | (2^32-1 - entry index)
  uint32_t* sbm;                 // [KW][32 W steps][dm, rm] bitmaps: the step's map holds the key
  uint32_t KW;                   // 32-key words per bitmap
  uint64_t* dm_excl;            // per chain FO entry: item prefix of the distinct-map table
  uint4* fo_rng;                // chain FO entries: leaf key ranges {lo0, n0, lo1, n1}
  uint64_t *tot;                // [0] dm items, [2] main FO chunks, [3] main shift chunks, [4] [3] + rm items
  uint8_t* out;
  uint32_t* err;
  uint32_t c_lo, c_hi;           // resolve / copy: chunks [c_lo, c_hi), c_lo a multiple of 32
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
//    The (checkpoint, count) pairs are read by the whole block and applied in
//    table order by one thread (a repeated checkpoint keeps its last count);
//    the prefix is a block scan (modulo 2^32, as the reference's uint32 sum).
__global__ void rrs_kernel(RArgs a) {
  __shared__ uint2 pairs[256];
  __shared__ uint64_t sh[33];
  for (uint32_t s = blockIdx.x; s < a.ndiff; s += gridDim.x) {
    const DiffInfo& d = a.di[s];
    uint32_t* r = a.rrs + d.rrs_begin;
    for (uint32_t j = threadIdx.x; j <= d.id; j += blockDim.x) r[j] = 0;
    __syncthreads();
    for (uint32_t i0 = 0; i0 < d.P; i0 += blockDim.x) {
      const uint32_t i = i0 + threadIdx.x;
      if (i < d.P && threadIdx.x < 256)
        pairs[threadIdx.x] = make_uint2(rd32(d.base + d.cnt_off + 8ull * i), rd32(d.base + d.cnt_off + 8ull * i + 4));
      __syncthreads();
      if (threadIdx.x == 0) {
        const uint32_t m = d.P - i0 < blockDim.x ? d.P - i0 : blockDim.x;
        for (uint32_t k = 0; k < m; k++) {
          const uint2 p = pairs[k];
          if (p.x > d.id) { atomicOr(a.err, DERR_RANGE); continue; }
          r[p.x] = p.y;
        }
      }
      __syncthreads();
    }
    uint64_t carry = 0;
    for (uint32_t j0 = 0; j0 <= d.id; j0 += blockDim.x) {
      const uint32_t j = j0 + threadIdx.x;
      const uint64_t v = j <= d.id ? r[j] : 0;
      uint64_t tot;
      const uint64_t ex = block_excl_scan(v, sh, &tot);
      if (j <= d.id) r[j] = (uint32_t)(carry + ex + v);
      carry += tot;
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
// and the main checkpoint's item total (its entries lead the list, so their
// prefix is fo_excl itself)
__global__ void clen_kernel(RArgs a) {
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < a.nfo; g += (uint64_t)gridDim.x * blockDim.x) {
    const DiffInfo& d = a.di[a.fo_seg[g]];
    a.fo_clen[g] = (uint32_t)(a.fo_excl[g] - a.fo_excl[d.fo_begin]);
    if (g + 1 == a.F0)
      a.tot[2] = a.fo_excl[g] + (a.approach == APPROACH_TREE ? num_leaf_descendents(a.fo_node[g], a.M) : 1);
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
__device__ __forceinline__ uint32_t upper_entry(const uint64_t* excl, uint32_t n, uint64_t item) {
  // last entry e with excl[e] <= item
  uint32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (excl[mid] <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The same search by one whole warp: each round compares 32 evenly spaced
// pivots and keeps the span after the last pivot not above `item`, so n
// entries take ceil(log32 n) rounds of one load per lane (excl[0] = 0).
__device__ __forceinline__ uint32_t warp_upper_entry(const uint64_t* excl, uint32_t n, uint64_t item) {
  const uint32_t lane = threadIdx.x & 31;
  uint32_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const uint32_t step = (hi - lo) / 32 + 1;
    const uint64_t p = (uint64_t)lo + (uint64_t)lane * step;
    const bool ok = p <= hi && excl[p] <= item;
    const uint32_t b = __ballot_sync(0xffffffffu, ok);
    lo += (31 - __clz(b)) * step;
    const uint64_t h2 = (uint64_t)lo + step - 1;
    if (h2 < hi) hi = (uint32_t)h2;
  }
  return lo;
}

// Items numbered by an exclusive prefix over entries are processed in tiles of
// kExpandTile per block: two warps find the tile's first and last entry, the
// entries in between (each owns at least one item, or the tile falls back to
// searches in global memory) are staged in shared memory, and every item
// finds its entry by a binary search there.
constexpr uint32_t kExpandTile = 2048;
template <uint32_t TILE = kExpandTile>
struct ExpandTile {
  uint64_t ex[TILE + 1];
  uint32_t e0, e1;
};
template <uint32_t TILE>
__device__ __forceinline__ void expand_stage(ExpandTile<TILE>& T, const uint64_t* excl, uint32_t n, uint64_t t0,
                                             uint64_t t1) {
  const uint32_t warp = threadIdx.x >> 5;
  if (warp < 2) {
    const uint32_t e = warp_upper_entry(excl, n, warp == 0 ? t0 : t1 - 1);
    if ((threadIdx.x & 31) == 0) (warp == 0 ? T.e0 : T.e1) = e;
  }
  __syncthreads();
  const uint32_t cnt = T.e1 - T.e0 + 1;
  if (cnt <= TILE + 1)
    for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) T.ex[i] = excl[T.e0 + i];
  __syncthreads();
}
// entry owning `item` and the item's position within it
template <uint32_t TILE>
__device__ __forceinline__ uint32_t expand_entry(const ExpandTile<TILE>& T, const uint64_t* excl, uint32_t n,
                                                 uint64_t item, uint64_t* j) {
  const uint32_t cnt = T.e1 - T.e0 + 1;
  if (cnt > TILE + 1) {
    const uint32_t k = upper_entry(excl, n, item);
    *j = item - excl[k];
    return k;
  }
  uint32_t lo = 0, hi = cnt - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (T.ex[mid] <= item) lo = mid; else hi = mid - 1;
  }
  *j = item - T.ex[lo];
  return T.e0 + lo;
}

// Tiles of two item lists taken in one grid: list 0's tiles first.
template <uint32_t TILE = kExpandTile>
struct TwoLists {
  uint64_t tot0, tot1, nt0, nt1;
  __device__ __forceinline__ TwoLists(uint64_t a0, uint64_t a1)
      : tot0(a0), tot1(a1), nt0((a0 + TILE - 1) / TILE), nt1((a1 + TILE - 1) / TILE) {}
  __device__ __forceinline__ uint64_t tiles() const { return nt0 + nt1; }
};

// main scatter: which entry writes node_list / copies each chunk last
// (src/tree_approach.cpp:825-925; ranks: FO entries 1+i, shift entries 2^32+i);
// the FO regions (prefix fo_excl, total tot[2]) and the shift regions (prefix
// sh_excl, total tot[3]) in one launch
// tiles of 256 items: the main checkpoint holds a few percent of the chunks,
// and tiles of 2048 left most SMs without one
constexpr uint32_t kCoverTile = 256;
__global__ void __launch_bounds__(256) main_cover_kernel(RArgs a) {
  __shared__ ExpandTile<kCoverTile> T;
  const TwoLists<kCoverTile> L(a.tot[2], a.tot[3]);
  const bool tree = a.approach == APPROACH_TREE;
  for (uint64_t tile = blockIdx.x; tile < L.tiles(); tile += gridDim.x) {
    const bool sh = tile >= L.nt0;
    const uint64_t total = sh ? L.tot1 : L.tot0;
    const uint64_t t0 = (sh ? tile - L.nt0 : tile) * kCoverTile;
    const uint64_t t1 = t0 + kCoverTile < total ? t0 + kCoverTile : total;
    const uint64_t* excl = sh ? a.sh_excl : a.fo_excl;
    const uint32_t n = sh ? a.S0 : a.F0;
    expand_stage(T, excl, n, t0, t1);
    for (uint64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
      uint64_t j64;
      const uint32_t i = expand_entry(T, excl, n, t, &j64);
      const uint32_t j = (uint32_t)j64;
      if (!sh) {
        uint64_t c = tree ? (uint64_t)(uint32_t)(leftmost_leaf(a.fo_node[i], a.M) - (a.N - 1) + j) : a.fo_node[i];
        if (c >= a.N) continue;
        const unsigned long long r = a.ntag | (1ull + i);
        atomicMax(reinterpret_cast<unsigned long long*>(&a.nl_rank[c]), r);
        atomicMax(reinterpret_cast<unsigned long long*>(&a.cp_rank[c]), r);
      } else {
        uint64_t c = tree ? (uint64_t)(uint32_t)(leftmost_leaf(a.sh_node[i], a.M) - (a.N - 1) + j) : a.sh_node[i];
        if (c >= a.N) continue;
        const unsigned long long r = a.ntag | ((1ull << 32) + i);
        atomicMax(reinterpret_cast<unsigned long long*>(&a.nl_rank[c]), r);
        if (a.sh_tree[i] == a.cur_main) atomicMax(reinterpret_cast<unsigned long long*>(&a.cp_rank[c]), r);
      }
    }
    __syncthreads();
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
    const uint64_t g = a.fo_cb + k;  // chain entries follow the main ones
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

// Chain table items are segments of up to kSegKeys consecutive keys of one
// entry, each handled by one thread.
constexpr uint32_t kSegKeys = 32;
__device__ __forceinline__ uint32_t segs_of(uint32_t keys) { return (keys + kSegKeys - 1) / kSegKeys; }

struct ChainDmCount {
  RArgs a;
  __device__ __forceinline__ uint64_t operator()(uint64_t k) const {
    const uint4 r = a.fo_rng[a.fo_cb + k];
    return (uint64_t)segs_of(r.y) + segs_of(r.w);
  }
};
struct ChainRmCount {
  RArgs a;
  __device__ __forceinline__ uint64_t operator()(uint64_t k) const {
    const uint64_t h = a.sh_cb + k;
    if (a.approach == APPROACH_LIST) return 1;
    const uint32_t node = a.sh_node[h];
    // repeat_map keys: the root (src/tree_approach.cpp:1069) and the leaf
    // range of num_leaf_descendents(node) from leftmost_leaf(node) (:1073-1078);
    // only keys in [N-1, M] can be looked up by a leaf
    uint64_t c = segs_of(num_leaf_descendents(node, a.M));
    if (node >= a.N - 1 && node <= a.M) c += 1;
    return c;
  }
};

// Items of every shift entry in one scan: the main checkpoint's regions
// (num_leaf_descendents(prev) chunks each), then the chain entries' repeat-map
// keys.  The main total goes to tot[3], the grand total to tot[4]; the chain
// items are numbered from tot[3] on.
struct ShiftItems {
  RArgs a;
  __device__ __forceinline__ uint64_t operator()(uint64_t h) const {
    if (h < a.S0) return a.approach == APPROACH_TREE ? num_leaf_descendents(a.sh_prev[h], a.M) : 1;
    return ChainRmCount{a}(h - a.sh_cb);
  }
};
struct StoreShiftExcl {
  RArgs a;
  __device__ __forceinline__ void operator()(uint64_t h, uint64_t ex, uint64_t v) const {
    a.sh_excl[h] = ex;
    if (h + 1 == a.S0) a.tot[3] = ex + v;
  }
};

__device__ __forceinline__ uint32_t key_of_leaf(const RArgs& a, uint32_t x) { return x - (a.N - 1); }

// The three entry scans of a restart in one pair of launches, each segment
// starting on a tile boundary and scanned on its own:
//   0: region length of every FO entry (FoLen) -> fo_excl
//   1: table segments of every chain FO entry, with its leaf ranges
//      (ChainDmCount, chain_ranges_kernel; the ranges are kept by the first
//      launch for the second) -> dm_excl, fo_rng, total tot[0]
//   2: items of every shift entry (ShiftItems) -> sh_excl, tot[3], total tot[4]
// Used when every segment fits the two-launch form (at most kReduceTiles
// tiles); otherwise the three scans run separately.
struct EntryScans {
  RArgs a;
  uint64_t n[3];
  uint32_t first[4];  // first tile of each segment; first[3] = all tiles
};
__device__ __forceinline__ uint4 chain_ranges_of(const RArgs& a, uint32_t g) {
  uint4 r = make_uint4(0, 0, 0, 0);
  if (a.approach == APPROACH_TREE) {
    uint32_t lo[2], hi[2];
    const int nr = fo_leaf_ranges(a.fo_node[g], a.N, a.M, lo, hi);
    if (nr > 0) { r.x = lo[0]; r.y = hi[0] - lo[0] + 1; }
    if (nr > 1) { r.z = lo[1]; r.w = hi[1] - lo[1] + 1; }
  } else {
    r.x = a.fo_node[g];
    r.y = 1;
  }
  return r;
}
// `ranges`: compute a chain entry's leaf ranges and keep them (first pass),
// or read the kept ones (second pass)
__device__ __forceinline__ uint64_t entry_scan_val(const EntryScans& e, int k, uint64_t i, bool ranges) {
  if (k == 0) return FoLen{e.a.fo_node, e.a.M, e.a.approach == APPROACH_TREE ? 1 : 0}(i);
  if (k == 1) {
    const uint32_t g = e.a.fo_cb + (uint32_t)i;
    uint4 r;
    if (ranges) {
      r = chain_ranges_of(e.a, g);
      e.a.fo_rng[g] = r;
    } else {
      r = e.a.fo_rng[g];
    }
    return (uint64_t)segs_of(r.y) + segs_of(r.w);
  }
  return ShiftItems{e.a}(i);
}
__device__ __forceinline__ int entry_scan_seg(const EntryScans& e, uint32_t b) {
  return b < e.first[1] ? 0 : b < e.first[2] ? 1 : 2;
}
__global__ void entry_scan_sums_kernel(EntryScans e, uint64_t* tile_sums) {
  __shared__ uint64_t sh[33];
  const int k = entry_scan_seg(e, blockIdx.x);
  const uint64_t base = (uint64_t)(blockIdx.x - e.first[k]) * kScanTile;
  uint64_t sum = 0;
  for (int q = 0; q < kScanPerThread; q++) {
    const uint64_t i = base + (uint64_t)q * kScanThreads + threadIdx.x;
    if (i < e.n[k]) sum += entry_scan_val(e, k, i, true);
  }
  uint64_t total;
  block_excl_scan(sum, sh, &total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}
__global__ void __launch_bounds__(kScanThreads, 3) entry_scan_emit_kernel(EntryScans e, const uint64_t* tile_sums) {
  __shared__ uint64_t sh[33];
  const int k = entry_scan_seg(e, blockIdx.x);
  uint64_t part = 0;
  for (uint32_t q = e.first[k] + threadIdx.x; q < blockIdx.x; q += blockDim.x) part += tile_sums[q];
  uint64_t off;
  block_excl_scan(part, sh, &off);
  const uint64_t base = (uint64_t)(blockIdx.x - e.first[k]) * kScanTile;
  uint64_t v[kScanPerThread];
  uint64_t sum = 0;
#pragma unroll
  for (int q = 0; q < kScanPerThread; q++) {
    const uint64_t i = base + (uint64_t)threadIdx.x * kScanPerThread + q;
    v[q] = i < e.n[k] ? entry_scan_val(e, k, i, false) : 0;
    sum += v[q];
  }
  uint64_t tile_total;
  uint64_t ex = block_excl_scan(sum, sh, &tile_total) + off;
  if (threadIdx.x == 0 && blockIdx.x + 1 == e.first[k + 1]) {
    if (k == 1) e.a.tot[0] = off + tile_total;
    if (k == 2) e.a.tot[4] = off + tile_total;
  }
#pragma unroll
  for (int q = 0; q < kScanPerThread; q++) {
    const uint64_t i = base + (uint64_t)threadIdx.x * kScanPerThread + q;
    if (i < e.n[k]) {
      if (k == 0) {
        e.a.fo_excl[i] = ex;
      } else if (k == 1) {
        e.a.dm_excl[i] = ex;
      } else {
        StoreShiftExcl{e.a}(i, ex, v[q]);
      }
    }
    ex += v[q];
  }
}

// Every (step, key) that a chain step's distinct map (FO entries) or repeat
// map (shift entries) holds, both entry lists in one launch, each entry cut
// into segments of up to kSegKeys consecutive keys (one thread each):
//   * distinct map: the key's position in the step's data section, by a plain
//     store: the FO entries of one diff are disjoint subtrees (or distinct
//     chunks), so no two segments of a step share a key;
//   * repeat map: the entry that the reference inserts first (the lowest
//     entry index; shift entries as 2h for the root key, 2h+1 for the leaf
//     keys) through an atomicMax of tag | (2^32-1 - index): the arithmetic
//     of num_leaf_descendents lets ranges of one step overlap when the leaf
//     count is not a power of two.  `tag` is this restart's epoch in the
//     high word, so a cell written by an earlier restart loses to any write
//     of this one and needs no clearing pass;
//   * per 32-key word, bitmaps of the steps' maps that hold each key
//     ([word][step][dm, rm], cleared for every restart): one or two atomicOr
//     per segment.
// A malformed chain whose FO entries of one step overlap gets one of them
// for the shared keys (the reference keeps the first).
__device__ __forceinline__ void seg_bits(const RArgs& a, uint32_t s, int d, uint32_t k0, uint32_t lo, uint32_t hi) {
  uint32_t* base = a.sbm + (uint64_t)s * 2 + d;
  const uint64_t stride = (uint64_t)a.W * 64;  // words per 32-key word row
  if (lo) atomicOr(base + (uint64_t)(k0 >> 5) * stride, lo);
  if (hi) atomicOr(base + (uint64_t)((k0 >> 5) + 1) * stride, hi);
}
constexpr uint32_t kChainTile = 256;
__global__ void __launch_bounds__(256) chain_tables_kernel(RArgs a) {
  // tiles of one segment per thread: many small tiles keep every SM busy
  // (the per-segment work is a chain of dependent loads)
  __shared__ ExpandTile<kChainTile> T;
  if (a.nsteps == 0) return;
  const uint64_t rbase = a.tot[3];  // repeat-map segments are numbered from here
  const TwoLists<kChainTile> L(a.tot[0], a.tot[4] - rbase);
  const bool tree = a.approach == APPROACH_TREE;
  const uint32_t leaf0 = a.N - 1;
  for (uint64_t tile = blockIdx.x; tile < L.tiles(); tile += gridDim.x) {
    const bool rm = tile >= L.nt0;
    const uint64_t total = rm ? L.tot1 : L.tot0, base = rm ? rbase : 0;
    const uint64_t t0 = (rm ? tile - L.nt0 : tile) * kChainTile;
    const uint64_t t1 = t0 + kChainTile < total ? t0 + kChainTile : total;
    const uint64_t* excl = rm ? a.sh_excl + a.sh_cb : a.dm_excl;
    const uint32_t n = rm ? a.nsh - a.sh_cb : a.nfo - a.fo_cb;
    // list and basic: every chain entry is exactly one item, so an item's
    // entry is its own index and nothing needs expanding
    if (tree) expand_stage(T, excl, n, base + t0, base + t1);
    const uint32_t lane = threadIdx.x & 31;
    // whole warps step together (the fast path below is a warp operation)
    for (uint64_t tw = t0 + (threadIdx.x & ~31u); tw < t1; tw += blockDim.x) {
      const uint64_t t = tw + lane;
      const bool in = t < t1;
      uint32_t k = 0, j = 0;
      if (in && tree) {
        uint64_t j64;
        k = expand_entry(T, excl, n, base + t, &j64);
        j = (uint32_t)j64;
      } else if (in) {
        k = (uint32_t)t;
      }
      uint32_t lo = 0, hi = 0, k0 = 0;
      if (!rm && tree) {
        // a distinct-map segment: leaves x0 .. x0 + cnt - 1 of entry g
        const uint32_t g = a.fo_cb + k;
        uint32_t s = 0, x0 = 0, cnt = 0, pos0 = 0;
        if (in) {
          s = a.fo_seg[g] - 1;
          const uint4 r = a.fo_rng[g];
          const uint32_t n0 = segs_of(r.y);
          x0 = j < n0 ? r.x + j * kSegKeys : r.z + (j - n0) * kSegKeys;
          const uint32_t left = j < n0 ? r.y - j * kSegKeys : r.w - (j - n0) * kSegKeys;
          cnt = left < kSegKeys ? left : kSegKeys;
          // position of leaf x in the step's data: fo_clen + x - leftmost leaf
          pos0 = a.fo_clen[g] + x0 - leftmost_leaf(a.fo_node[g], a.M);
        }
        k0 = x0 - leaf0;
        // 32 full, 32-key aligned, consecutive segments of one entry (the
        // large regions): the warp writes them together, coalesced, and sets
        // whole bitmap words
        const uint32_t g0 = __shfl_sync(0xffffffffu, g, 0), k00 = __shfl_sync(0xffffffffu, k0, 0);
        const bool uni = __all_sync(0xffffffffu, in && cnt == kSegKeys && (k0 & 31) == 0 && g == g0 &&
                                                   k0 == k00 + kSegKeys * lane);
        if (uni) {
          const uint32_t p00 = __shfl_sync(0xffffffffu, pos0, 0);
          uint32_t* cell = a.dm_off + (uint64_t)s * a.K + k00;
#pragma unroll 4
          for (uint32_t q = 0; q < kSegKeys; q++) cell[q * 32 + lane] = p00 + q * 32 + lane;
          atomicOr(a.sbm + (uint64_t)((k00 >> 5) + lane) * a.W * 64 + (uint64_t)s * 2, ~0u);
          continue;
        }
        if (!in) continue;
        uint32_t* cell = a.dm_off + (uint64_t)s * a.K;
        for (uint32_t q = 0; q < cnt; q++) cell[k0 + q] = pos0 + q;
        const uint64_t m = (cnt == 32 ? ~0ull >> 32 : ((1ull << cnt) - 1)) << (k0 & 31);
        seg_bits(a, s, 0, k0, (uint32_t)m, (uint32_t)(m >> 32));
        continue;
      }
      if (!in) continue;
      if (!rm) {
        // list / basic: one chunk per entry
        const uint32_t g = a.fo_cb + k;
        const uint32_t s = a.fo_seg[g] - 1;
        const uint4 r = a.fo_rng[g];
        if (r.x >= a.N) continue;
        k0 = r.x;
        a.dm_off[(uint64_t)s * a.K + k0] = a.fo_clen[g];
        lo = 1u << (k0 & 31);
        seg_bits(a, s, 0, k0, lo, hi);
      } else {
        const uint32_t h = a.sh_cb + k;
        const uint32_t s = a.sh_seg[h] - 1;
        unsigned long long* cell = reinterpret_cast<unsigned long long*>(a.rm_tab + (uint64_t)s * a.K);
        if (!tree) {
          k0 = a.sh_node[h];
          if (k0 >= a.N) continue;
          atomicMax(cell + k0, a.tag | (0xffffffffull - 2ull * h));
          lo = 1u << (k0 & 31);
        } else {
          const uint32_t node = a.sh_node[h];
          const uint32_t len = num_leaf_descendents(node, a.M);
          const uint32_t nseg = segs_of(len);
          uint32_t x0, cnt;
          unsigned long long v;
          if (j < nseg) {
            x0 = leftmost_leaf(node, a.M) + j * kSegKeys;
            cnt = len - j * kSegKeys < kSegKeys ? len - j * kSegKeys : kSegKeys;
            v = a.tag | (0xffffffffull - (2ull * h + 1));
          } else {
            x0 = node;
            cnt = 1;
            v = a.tag | (0xffffffffull - 2ull * h);
          }
          // keys of the segment in [N-1, M]; they span at most two words
          uint32_t a0 = x0 > leaf0 ? x0 : leaf0;
          uint64_t a1 = (uint64_t)x0 + cnt;  // exclusive
          if (a1 > (uint64_t)a.M + 1) a1 = (uint64_t)a.M + 1;
          if ((uint64_t)a0 >= a1) continue;
          k0 = x0 >= leaf0 ? x0 - leaf0 : 0;
          for (uint32_t x = a0; x < (uint32_t)a1; x++) {
            const uint32_t key = x - leaf0;
            atomicMax(cell + key, v);
            if ((key >> 5) == (k0 >> 5)) lo |= 1u << (key & 31);
            else hi |= 1u << (key & 31);
          }
        }
        seg_bits(a, s, 1, k0, lo, hi);
      }
    }
    if (tree) __syncthreads();
  }
}

// 32 x 32 bit transpose across a warp: lane i holds row i on entry, column
// `lane` on return (bit i of the result = bit `lane` of row i).
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int r = 0; r < 5; r++) {
    const uint32_t jj = 16u >> r, m = masks[r];
    const uint32_t y = __shfl_xor_sync(0xffffffffu, x, jj);
    x = (lane & jj) ? ((x & ~m) | ((y >> jj) & m)) : ((x & m) | ((y << jj) & ~m));
  }
  return x;
}

// Masks of the warp's own 32 keys for the first 32 steps, by one coalesced
// load and a transpose; lane l gets key 32w + l (the chunk's own key).
struct OwnMasks {
  uint32_t key;  // the key they belong to
  uint2 m;       // {dm, rm} bits of steps 0..31
};

// The {dm, rm} bits of `key` at step s (one word pair of its 32-key row).
__device__ __forceinline__ uint32_t key_bits(const RArgs& a, uint32_t key, uint32_t s) {
  const uint2 v = reinterpret_cast<const uint2*>(a.sbm)[((uint64_t)(key >> 5) * a.W * 32) + s];
  const uint32_t b = key & 31;
  return ((v.x >> b) & 1u) | (((v.y >> b) & 1u) << 1);
}

// The first step at or after s whose distinct (bit 0) or repeat (bit 1) map
// holds `key`: from the warp's own masks, or by probing the key's row step by
// step (a key reached through a shifted duplicate).  nsteps when none.
__device__ __forceinline__ uint32_t next_step(const RArgs& a, const OwnMasks& own, uint32_t key, uint32_t s,
                                              bool* in_dm) {
  if (key == own.key && a.nsteps <= 32) {
    const uint32_t m = (own.m.x | own.m.y) & (s < 32 ? ~0u << s : 0u);
    if (!m) return a.nsteps;
    const uint32_t f = __ffs(m) - 1;
    *in_dm = (own.m.x >> f) & 1u;
    return f;
  }
  for (; s < a.nsteps; s++) {
    const uint32_t b = key_bits(a, key, s);
    if (b) {
      *in_dm = b & 1u;
      return s;
    }
  }
  return a.nsteps;
}

// entry index stored in a repeat-map cell
__device__ __forceinline__ uint32_t cell_index(uint64_t v) { return 0xffffffffu - (uint32_t)v; }

// offset of leaf/chunk x (key `key`) in step s's data through its distinct
// map (the caller has seen the step's mask bit for the key)
__device__ __forceinline__ uint64_t chain_dm_offset(const RArgs& a, uint32_t s, uint32_t key) {
  return (uint64_t)a.dm_off[(uint64_t)s * a.K + key] * a.cs;
}
__device__ __forceinline__ bool dm_has(const RArgs& a, uint32_t s, uint32_t key) {
  return key_bits(a, key, s) & 1u;
}

// 4. where chunk c's bytes come from: node_list and the first copy source
//    after the main checkpoint (src/tree_approach.cpp:825-937), then the walk
//    down the chain (src/tree_approach.cpp:1083-1118,
//    src/list_approach.cpp:520-567, src/basic_approach.cpp:293-312).
//    seg 0 is the main diff; off = kNone: the reference writes nothing.
__device__ __forceinline__ void resolve_chunk(const RArgs& a, const OwnMasks& own, uint64_t c, uint32_t& seg,
                                              uint64_t& off) {
  const uint32_t cur = a.cur_main;
  const bool tree = a.approach == APPROACH_TREE;
  const uint64_t nr0 = a.nl_rank[c], cr0 = a.cp_rank[c];
  const uint64_t nr = nr0 >= a.ntag ? nr0 - a.ntag : 0, cr = cr0 >= a.ntag ? cr0 - a.ntag : 0;
  uint32_t x, t;
  if (nr == 0) {
    // "same as previous" (src/tree_approach.cpp:932-937)
    x = tree ? (uint32_t)c + a.N - 1 : (uint32_t)c;
    t = cur - 1;
  } else if (nr < (1ull << 32)) {
    x = (uint32_t)c;
    t = cur;
  } else {
    const uint32_t i = (uint32_t)(nr - (1ull << 32));
    if (tree) {
      const uint32_t j = (uint32_t)c - (leftmost_leaf(a.sh_node[i], a.M) - (a.N - 1));
      x = leftmost_leaf(a.sh_prev[i], a.M) + j;
    } else {
      x = a.sh_prev[i];
    }
    t = a.sh_tree[i];
  }
  seg = 0;
  off = kNone;
  if (cr != 0) {
    uint64_t res;
    if (cr < (1ull << 32)) {
      const uint32_t i = (uint32_t)(cr - 1);
      const uint64_t base = tree ? (uint64_t)a.fo_clen[i] * a.cs : (uint64_t)i * a.cs;
      const uint64_t within = tree ? (c - (leftmost_leaf(a.fo_node[i], a.M) - (a.N - 1))) * (uint64_t)a.cs : 0;
      res = base + within;
    } else {
      const uint32_t i = (uint32_t)(cr - (1ull << 32));
      const uint64_t within = tree ? (c - (leftmost_leaf(a.sh_node[i], a.M) - (a.N - 1))) * (uint64_t)a.cs : 0;
      res = a.sh_off[i] + within;
    }
    if (res < (1ull << kOffBits)) off = res;
  }
  if (a.nsteps == 0) return;
  const uint32_t id0 = cur - 1;                // id of step 0
  const uint32_t idl = id0 - (a.nsteps - 1);  // id of the last step
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
    bool in_dm = false;
    const uint32_t found = next_step(a, own, key, id0 - t, &in_dm);
    if (found >= a.nsteps) break;  // never mentioned again: left as is
    const uint32_t s = found;
    const uint32_t ts = id0 - s;
    if (in_dm) {
      const uint64_t o = chain_dm_offset(a, s, key);
      if (o < (1ull << kOffBits)) { seg = 1 + s; off = o; }
      break;
    }
    if (a.approach == APPROACH_BASIC) break;
    const uint32_t r = cell_index(a.rm_tab[(uint64_t)s * a.K + key]);
    const uint32_t h = r >> 1;
    uint32_t pnode;
    const uint32_t ptree = a.sh_tree[h];
    if (tree && (r & 1)) pnode = leftmost_leaf(a.sh_prev[h], a.M) + (x - leftmost_leaf(a.sh_node[h], a.M));
    else pnode = a.sh_prev[h];
    if (ptree == ts) {
      uint32_t pkey = 0;
      bool ok;
      if (tree) {
        ok = pnode >= a.N - 1 && pnode <= a.M;
        if (ok) pkey = key_of_leaf(a, pnode);
      } else {
        ok = pnode < a.N;
        pkey = pnode;
      }
      if (ok && dm_has(a, s, pkey)) {
        const uint64_t o2 = chain_dm_offset(a, s, pkey);
        if (o2 < (1ull << kOffBits)) { seg = 1 + s; off = o2; }
      }
      break;
    }
    x = pnode;
    t = ptree;
  }
}

// 5. Each warp copies its 32 chunks: lane q holds chunk q's source and byte
//    count, and the warp moves the chunks' 16-byte units with every lane busy
//    (unit f of the tile is chunk f / units-per-chunk).  A source that is not
//    16-byte aligned (diff data sections are only 4-byte aligned) is read as
//    aligned 16-byte words, the word after a unit taken from the next lane,
//    and the unit is cut out with funnel shifts; every load stays inside a
//    16-byte word holding at least one byte of the source region.
__device__ __forceinline__ uint4 cut16(const uint4& w0, const uint4& w1, uint32_t d) {
  uint32_t v[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
  uint32_t o[5];
  const uint32_t sh = (d & 3) * 8;
  switch (d >> 2) {
    case 0: o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; o[3] = v[3]; o[4] = v[4]; break;
    case 1: o[0] = v[1]; o[1] = v[2]; o[2] = v[3]; o[3] = v[4]; o[4] = v[5]; break;
    case 2: o[0] = v[2]; o[1] = v[3]; o[2] = v[4]; o[3] = v[5]; o[4] = v[6]; break;
    default: o[0] = v[3]; o[1] = v[4]; o[2] = v[5]; o[3] = v[6]; o[4] = v[7]; break;
  }
  if (sh == 0) return make_uint4(o[0], o[1], o[2], o[3]);
  return make_uint4(__funnelshift_r(o[0], o[1], sh), __funnelshift_r(o[1], o[2], sh), __funnelshift_r(o[2], o[3], sh),
                    __funnelshift_r(o[3], o[4], sh));
}
constexpr int kCopyUnroll = 4;
__device__ __forceinline__ void copy_tile(const RArgs& a, uint64_t c0, const uint8_t* src, uint32_t nb) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t cs = a.cs;
  const unsigned long long sp = reinterpret_cast<unsigned long long>(src);
  uint8_t* out0 = a.out + c0 * cs;
  if ((cs & 15) != 0 || (reinterpret_cast<uintptr_t>(a.out) & 15) != 0) {
    // byte by byte (odd chunk sizes)
    const uint64_t total = (uint64_t)cs * 32;
    for (uint64_t f = lane; f < total; f += 32) {
      const uint32_t q = (uint32_t)(f / cs), b = (uint32_t)(f - (uint64_t)q * cs);
      const uint8_t* s = reinterpret_cast<const uint8_t*>(__shfl_sync(0xffffffffu, sp, q));
      const uint32_t n = __shfl_sync(0xffffffffu, nb, q);
      if (b < n) out0[(uint64_t)q * cs + b] = s[b];
    }
    return;
  }
  const uint32_t upc = cs >> 4;
  const int lg = (upc & (upc - 1)) == 0 ? __ffs(upc) - 1 : -1;
  const uint64_t total = (uint64_t)upc * 32;
  for (uint64_t f0 = 0; f0 < total; f0 += 32 * kCopyUnroll) {
    uint4 w0[kCopyUnroll], w1[kCopyUnroll];
    uint32_t qv[kCopyUnroll], byte[kCopyUnroll], m[kCopyUnroll], dv[kCopyUnroll];
    bool own1[kCopyUnroll];
#pragma unroll
    for (int k = 0; k < kCopyUnroll; k++) {
      const uint64_t f = f0 + (uint64_t)k * 32 + lane;
      const bool in = f < total;
      const uint32_t q = in ? (lg >= 0 ? (uint32_t)(f >> lg) : (uint32_t)(f / upc)) : 31;
      const uint32_t u = in ? (uint32_t)(f - (uint64_t)q * upc) : 0;
      const unsigned long long s = __shfl_sync(0xffffffffu, sp, q);
      const uint32_t n = __shfl_sync(0xffffffffu, nb, q);
      const uint32_t b = u * 16;
      const uint32_t mm = in && b < n ? (n - b < 16 ? n - b : 16) : 0;
      const uint32_t d = (uint32_t)(s & 15);
      const unsigned long long A = s - d;
      // the next unit's lane holds the following word when it is in the same
      // chunk and live; otherwise this lane reads that word itself
      const bool need1 = mm && d + mm > 16;
      const bool next_live = lane < 31 && u + 1 < upc && b + 16 < n;
      own1[k] = need1 && !next_live;
      w0[k] = mm ? __ldcs(reinterpret_cast<const uint4*>(A + b)) : make_uint4(0, 0, 0, 0);
      w1[k] = own1[k] ? __ldcs(reinterpret_cast<const uint4*>(A + b + 16)) : make_uint4(0, 0, 0, 0);
      qv[k] = q;
      byte[k] = b;
      m[k] = mm;
      dv[k] = d;
    }
#pragma unroll
    for (int k = 0; k < kCopyUnroll; k++) {
      uint4 nx;
      nx.x = __shfl_down_sync(0xffffffffu, w0[k].x, 1);
      nx.y = __shfl_down_sync(0xffffffffu, w0[k].y, 1);
      nx.z = __shfl_down_sync(0xffffffffu, w0[k].z, 1);
      nx.w = __shfl_down_sync(0xffffffffu, w0[k].w, 1);
      if (!m[k]) continue;
      const uint4 v = dv[k] == 0 ? w0[k] : cut16(w0[k], own1[k] ? w1[k] : nx, dv[k]);
      uint8_t* dst = out0 + (uint64_t)qv[k] * cs + byte[k];
      if (m[k] == 16) {
        *reinterpret_cast<uint4*>(dst) = v;
      } else {
        for (uint32_t i = 0; i < m[k]; i++) {
          const uint32_t w = i < 4 ? v.x : i < 8 ? v.y : i < 12 ? v.z : v.w;
          dst[i] = (uint8_t)(w >> ((i & 3) * 8));
        }
      }
    }
  }
}

// Where chunk c of a tile comes from: a source address and byte count (0:
// the chunk is not written).
__device__ __forceinline__ void chunk_source(const RArgs& a, const OwnMasks& own, uint64_t c, const uint8_t*& src,
                                             uint32_t& nb) {
  src = nullptr;
  nb = 0;
  if (c >= a.N) return;
  uint32_t seg;
  uint64_t off;
  resolve_chunk(a, own, c, seg, off);
  if (off == kNone) return;
  const DiffInfo& d = a.di[seg];
  const uint64_t o = d.data_off + off;
  if (o >= d.len) return;
  uint64_t n = a.cs;
  const uint64_t left = a.datalen - c * a.cs;
  if (n > left) n = left;
  if (n > d.len - o) n = d.len - o;
  src = d.base + o;
  nb = (uint32_t)n;
}

// 4. Every chunk's source address and byte count, in a pass of its own: the
// walks' dependent loads want all the warps an SM can hold, the copy wants
// bytes in flight per warp.
// Whole warps take 32 consecutive chunks at a time: the warp's own keys'
// step masks come from one coalesced load and a transpose per 32 steps.
__global__ void __launch_bounds__(256, 8) resolve_kernel(RArgs a) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint2* bm = reinterpret_cast<const uint2*>(a.sbm);
  for (uint64_t cw = a.c_lo + (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); cw < a.c_hi; cw += stride) {
    const uint64_t c = cw + lane;
    OwnMasks own;
    own.key = (uint32_t)c;  // chunk c's own key (tree: leaf N-1+c, list: chunk c)
    own.m = make_uint2(0, 0);
    if (a.nsteps) {
      const uint32_t st = lane;
      const uint2 v = st < a.nsteps ? bm[(cw >> 5) * a.W * 32 + st] : make_uint2(0, 0);
      own.m = make_uint2(warp_transpose32(v.x), warp_transpose32(v.y));
    }
    if (c < a.c_hi) {
      const uint8_t* src;
      uint32_t nb;
      chunk_source(a, own, c, src, nb);
      a.srcp[c] = reinterpret_cast<uint64_t>(src);
      a.nbv[c] = nb;
    }
  }
}

// 5. Each warp copies 32 consecutive chunks from the sources resolved above.
__global__ void __launch_bounds__(256, 3) restore_copy_kernel(RArgs a) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t t_hi = ((uint64_t)a.c_hi + 31) / 32;
  for (uint64_t wt = a.c_lo / 32 + (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); wt < t_hi;
       wt += warps) {
    const uint64_t c = wt * 32 + lane;
    const uint8_t* src = nullptr;
    uint32_t nb = 0;
    if (c < a.c_hi) {
      src = reinterpret_cast<const uint8_t*>(a.srcp[c]);
      nb = a.nbv[c];
    }
    copy_tile(a, wt * 32, src, nb);
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

// One wave of resolve_kernel: its CTAs do equal work, so a grid of 1.33
// waves (eight CTAs per SM asked, six resident) would run its last third on
// a third of the GPU.
static uint32_t resolve_grid() {
  static const uint32_t g = [] {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, resolve_kernel, 256, 0) != cudaSuccess || per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    }
    return (uint32_t)(num_sms() * per_sm);
  }();
  return g;
}

// Chunk ranges the resolve and copy passes can be pipelined over
// (MTCHECK_RESTART_PARTS, 1-7; one below 2^16 chunks).  One by default: with
// resolve in one wave, four ranges measured 0.690 ms against 0.683 ms for
// one at 1 GiB / 256 B (the copy already holds every SM).
static uint32_t restart_parts(uint32_t N) {
  static int v = [] {
    const char* e = std::getenv("MTCHECK_RESTART_PARTS");
    const int x = e ? std::atoi(e) : 1;
    return x < 1 ? 1 : x > 7 ? 7 : x;
  }();
  return N < (1u << 16) ? 1 : (uint32_t)v;
}

// Restart scratch owned by the engine between calls.
struct RestartScratch {
  DevBuf<DiffInfo> di;
  DevBuf<uint32_t> fo_node, fo_seg, fo_clen, sh_node, sh_prev, sh_tree, sh_seg, rrs, fo_at, dm_off, sbm;
  DevBuf<uint64_t> fo_excl, sh_off, sh_excl, nl_rank, cp_rank, dm_excl, tot, scan, scan_total, rm_tab, srcp;
  DevBuf<uint32_t> nbv;
  DevBuf<uint4> fo_rng;
  // epochs: repeat-map cells and the main scatter ranks hold the epoch of
  // the restart that wrote them; the three buffers are zeroed when one of
  // them is (re)allocated or the epoch reaches 2^30
  uint32_t epoch = 0;
  const void* seen[4] = {nullptr, nullptr, nullptr, nullptr};
};

void destroy_restart_scratch(RestartScratch* r) { delete r; }

// Headers of up to kHeaderBatch diffs per launch, one thread per byte (the
// diffs may start at any address).
constexpr uint32_t kHeaderBatch = 64;
struct HeaderSrc {
  const uint8_t* p[kHeaderBatch];
  uint64_t len[kHeaderBatch];
  uint32_t n;
};
static __global__ void header_gather_kernel(HeaderSrc s, uint8_t* out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t k = t / (uint32_t)sizeof(HeaderHost), b = t % (uint32_t)sizeof(HeaderHost);
  if (k >= s.n) return;
  out[t] = s.len[k] >= sizeof(HeaderHost) && s.p[k] ? s.p[k][b] : 0;
}

int Engine::read_headers(const std::vector<const uint8_t*>& ptrs, const std::vector<uint64_t>& lens,
                         std::vector<HeaderHost>& out) {
  const size_t n = ptrs.size(), bytes = n * sizeof(HeaderHost);
  out.assign(n, HeaderHost{});
  if (n == 0) return ST_OK;
  MTC_CUDA_R(hdr_dev_.ensure(bytes, stream_));
  if (hdr_host_cap_ < bytes) {
    // grown geometrically, as the descriptors below
    const size_t cap = std::max<size_t>({bytes, 2 * hdr_host_cap_, 16u << 10});
    if (hdr_host_) cudaFreeHost(hdr_host_);
    hdr_host_ = nullptr;
    hdr_host_cap_ = 0;
    MTC_CUDA_R(cudaMallocHost(reinterpret_cast<void**>(&hdr_host_), cap));
    hdr_host_cap_ = cap;
  }
  for (size_t i0 = 0; i0 < n; i0 += kHeaderBatch) {
    HeaderSrc src{};
    src.n = (uint32_t)std::min<size_t>(kHeaderBatch, n - i0);
    for (uint32_t k = 0; k < src.n; k++) {
      src.p[k] = ptrs[i0 + k];
      src.len[k] = lens[i0 + k];
    }
    const uint32_t threads = src.n * (uint32_t)sizeof(HeaderHost);
    header_gather_kernel<<<(threads + 255) / 256, 256, 0, stream_>>>(src, hdr_dev_.p + i0 * sizeof(HeaderHost));
    note_launch();
    MTC_CUDA_R(cudaGetLastError());
  }
  MTC_CUDA_R(cudaMemcpyAsync(hdr_host_, hdr_dev_.p, bytes, cudaMemcpyDeviceToHost, stream_));
  MTC_CUDA_R(cudaStreamSynchronize(stream_));
  std::memcpy(out.data(), hdr_host_, bytes);
  return ST_OK;
}

uint64_t Engine::restart_scratch_bytes() const {
  if (!rs_) return restart_stage.n;
  const RestartScratch& R = *rs_;
  uint64_t b = restart_stage.n + sizeof(DiffInfo) * R.di.n + sizeof(uint4) * R.fo_rng.n;
  for (const auto* x : {&R.fo_node, &R.fo_seg, &R.fo_clen, &R.sh_node, &R.sh_prev, &R.sh_tree, &R.sh_seg, &R.rrs,
                        &R.fo_at, &R.dm_off, &R.sbm, &R.nbv})
    b += sizeof(uint32_t) * x->n;
  for (const auto* x : {&R.fo_excl, &R.sh_off, &R.sh_excl, &R.nl_rank, &R.cp_rank, &R.dm_excl, &R.tot, &R.scan,
                        &R.scan_total, &R.rm_tab, &R.srcp})
    b += sizeof(uint64_t) * x->n;
  return b;
}

static void set_scratch_pool(RestartScratch* r, cudaMemPool_t pool) {
  r->di.pool = pool;
  r->fo_rng.pool = pool;
  for (auto* b : {&r->fo_node, &r->fo_seg, &r->fo_clen, &r->sh_node, &r->sh_prev, &r->sh_tree, &r->sh_seg, &r->rrs,
                  &r->fo_at, &r->dm_off, &r->sbm})
    b->pool = pool;
  for (auto* b : {&r->fo_excl, &r->sh_off, &r->sh_excl, &r->nl_rank, &r->cp_rank, &r->dm_excl, &r->tot,
                  &r->scan, &r->scan_total, &r->rm_tab, &r->srcp})
    b->pool = pool;
  r->nbv.pool = pool;
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
    // entry indices are 32-bit on the device, shift entries doubled in the
    // table cells (2h + 1)
    if ((uint64_t)nfo + d.F >= 0xffffffffull || (uint64_t)nsh + d.S >= (1ull << 31) ||
        (uint64_t)nrrs + d.id + 1 >= 0xffffffffull)
      return fail(ST_ENOTSUP, "restart chain holds too many entries");
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
  StepTimer t_alloc("restart: table allocations", N);
  MTC_CUDA_R(R.di.ensure(di.size(), s));
  // the chain descriptors go up from pinned memory: a copy from pageable
  // memory would first wait for everything already on the stream
  StepTimer t_up("restart: descriptor upload", N);
  const size_t di_bytes = sizeof(DiffInfo) * di.size();
  if (rdi_ev_) MTC_CUDA_R(cudaEventSynchronize(rdi_ev_));  // the previous restart's copy has read it
  else MTC_CUDA_R(cudaEventCreateWithFlags(&rdi_ev_, cudaEventDisableTiming));
  if (rdi_host_bytes_ < di_bytes) {
    // grown geometrically: a chain grows by one diff per checkpoint, and
    // freeing pinned memory waits for the whole device
    const size_t cap = std::max<size_t>({di_bytes, 2 * rdi_host_bytes_, 64u << 10});
    if (rdi_host_) cudaFreeHost(rdi_host_);
    rdi_host_ = nullptr;
    rdi_host_bytes_ = 0;
    MTC_CUDA_R(cudaMallocHost(&rdi_host_, cap));
    rdi_host_bytes_ = cap;
  }
  std::memcpy(rdi_host_, di.data(), di_bytes);
  MTC_CUDA_R(cudaMemcpyAsync(R.di.p, rdi_host_, di_bytes, cudaMemcpyHostToDevice, s));
  MTC_CUDA_R(cudaEventRecord(rdi_ev_, s));
  MTC_CUDA_R(R.fo_node.ensure(nfo + 1, s));
  MTC_CUDA_R(R.fo_seg.ensure(nfo + 1, s));
  MTC_CUDA_R(R.fo_rng.ensure(nfo + 1, s));
  MTC_CUDA_R(R.fo_clen.ensure(nfo + 1, s));
  MTC_CUDA_R(R.fo_excl.ensure(nfo + 1, s));
  MTC_CUDA_R(R.sh_node.ensure(nsh + 1, s));
  MTC_CUDA_R(R.sh_prev.ensure(nsh + 1, s));
  MTC_CUDA_R(R.sh_tree.ensure(nsh + 1, s));
  MTC_CUDA_R(R.sh_seg.ensure(nsh + 1, s));
  MTC_CUDA_R(R.sh_off.ensure(nsh + 1, s));
  MTC_CUDA_R(R.sh_excl.ensure(nsh + 1, s));
  MTC_CUDA_R(R.rrs.ensure(nrrs + 1, s));
  MTC_CUDA_R(R.nl_rank.ensure(N, s));
  MTC_CUDA_R(R.cp_rank.ensure(N, s));
  MTC_CUDA_R(R.srcp.ensure(N, s));
  MTC_CUDA_R(R.nbv.ensure(N, s));
  MTC_CUDA_R(R.fo_at.ensure((size_t)M + 2, s));
  MTC_CUDA_R(R.dm_excl.ensure(nfo + 1, s));
  MTC_CUDA_R(R.tot.ensure(5, s));
  const uint32_t KW = (K + 31) / 32;
  MTC_CUDA_R(R.dm_off.ensure((size_t)std::max<uint32_t>(nsteps, 1) * K, s));
  MTC_CUDA_R(R.rm_tab.ensure((size_t)std::max<uint32_t>(nsteps, 1) * K, s));
  MTC_CUDA_R(R.sbm.ensure((size_t)KW * W * 32 * 2, s));
  if (R.rm_tab.p != R.seen[1] || R.nl_rank.p != R.seen[2] || R.cp_rank.p != R.seen[3] ||
      R.epoch >= (1u << 30) - 1) {
    MTC_CUDA_R(cudaMemsetAsync(R.rm_tab.p, 0, sizeof(uint64_t) * R.rm_tab.n, s));
    MTC_CUDA_R(cudaMemsetAsync(R.nl_rank.p, 0, sizeof(uint64_t) * R.nl_rank.n, s));
    MTC_CUDA_R(cudaMemsetAsync(R.cp_rank.p, 0, sizeof(uint64_t) * R.cp_rank.n, s));
    R.seen[1] = R.rm_tab.p;
    R.seen[2] = R.nl_rank.p;
    R.seen[3] = R.cp_rank.p;
    R.epoch = 0;
  }
  R.epoch++;
  const uint64_t scan_n = std::max<uint64_t>(nfo, nsh) + 1;
  // tile sums: one scan at a time, or the three entry scans side by side
  MTC_CUDA_R(R.scan.ensure(3 * (scan_n / kScanTile + 2), s));
  MTC_CUDA_R(R.scan_total.ensure(1, s));
  MTC_CUDA_R(err_.ensure(1, s));
  MTC_CUDA_R(cudaMemsetAsync(err_.p, 0, sizeof(uint32_t), s));

  RArgs a{};
  a.approach = approach;
  a.N = N; a.M = M; a.cs = cs; a.datalen = H.datalen;
  a.ndiff = (uint32_t)di.size(); a.nsteps = nsteps; a.W = W; a.K = K; a.cur_main = H.chkpt_id;
  a.di = R.di.p;
  a.nfo = nfo; a.nsh = nsh;
  a.F0 = di[0].F; a.S0 = di[0].S;
  a.fo_cb = di.size() > 1 ? di[1].fo_begin : nfo;
  a.sh_cb = di.size() > 1 ? di[1].sh_begin : nsh;
  a.tag = (uint64_t)R.epoch << 32;
  a.ntag = (uint64_t)R.epoch << 34;
  a.fo_node = R.fo_node.p; a.fo_seg = R.fo_seg.p; a.fo_clen = R.fo_clen.p; a.fo_excl = R.fo_excl.p;
  a.sh_node = R.sh_node.p; a.sh_prev = R.sh_prev.p; a.sh_tree = R.sh_tree.p; a.sh_seg = R.sh_seg.p;
  a.sh_off = R.sh_off.p; a.sh_excl = R.sh_excl.p;
  a.rrs = R.rrs.p;
  a.nl_rank = R.nl_rank.p; a.cp_rank = R.cp_rank.p;
  a.srcp = R.srcp.p; a.nbv = R.nbv.p;
  a.fo_at = R.fo_at.p;
  a.dm_off = R.dm_off.p; a.rm_tab = R.rm_tab.p; a.sbm = R.sbm.p; a.KW = KW;
  a.dm_excl = R.dm_excl.p; a.tot = R.tot.p;
  a.fo_rng = R.fo_rng.p;
  a.out = dev_out; a.err = err_.p;
  const bool tree = approach == APPROACH_TREE;

  // The second stream: clears that depend on nothing run there at once; the
  // chain tables run there beside the main checkpoint's scatter; each range
  // of resolved chunks is copied there while the next range is resolved.
  if (!rside_) {
    MTC_CUDA_R(cudaStreamCreateWithFlags(&rside_, cudaStreamNonBlocking));
    for (auto& e : rev_) MTC_CUDA_R(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  cudaStream_t side = rside_;
  StepTimer t_fork("restart: fork and clears", N);
  MTC_CUDA_R(cudaEventRecord(rev_[0], s));  // after the allocations and the previous restart
  MTC_CUDA_R(cudaStreamWaitEvent(side, rev_[0], 0));
  MTC_CUDA_R(cudaMemsetAsync(R.fo_at.p, 0xff, sizeof(uint32_t) * ((size_t)M + 2), side));
  if (nsteps) MTC_CUDA_R(cudaMemsetAsync(R.sbm.p, 0, sizeof(uint32_t) * (size_t)KW * W * 32 * 2, side));
  MTC_CUDA_R(cudaEventRecord(rev_[1], side));

  // 1-3: decode entries, repeat tables, source checkpoints
  StepTimer t_dec("restart: entry launches", N);
  MTC_CUDA_R(cudaMemsetAsync(R.tot.p, 0, sizeof(uint64_t) * 5, s));
  if (nfo + nsh) { load_entries_kernel<<<gsz((uint64_t)nfo + nsh), 256, 0, s>>>(a); note_launch(); }
  rrs_kernel<<<gsz(di.size(), 1, 4), 256, 0, s>>>(a);
  note_launch();
  if (nsh) { shift_tree_kernel<<<gsz(nsh), 256, 0, s>>>(a); note_launch(); }
  const uint32_t nfo_chain = nsteps ? nfo - a.fo_cb : 0;
  const uint64_t tiles[3] = {(nfo + kScanTile - 1) / kScanTile, (nfo_chain + kScanTile - 1) / kScanTile,
                             (nsh + kScanTile - 1) / kScanTile};
  const bool fused = tiles[0] <= reduce_tile_limit() && tiles[1] <= reduce_tile_limit() &&
                     tiles[2] <= reduce_tile_limit() && tiles[0] + tiles[1] + tiles[2] > 0;
  if (fused) {
    // the three entry scans in one pair of launches
    EntryScans e{a, {nfo, nfo_chain, nsh}, {0, (uint32_t)tiles[0], (uint32_t)(tiles[0] + tiles[1]),
                                            (uint32_t)(tiles[0] + tiles[1] + tiles[2])}};
    entry_scan_sums_kernel<<<e.first[3], kScanThreads, 0, s>>>(e, R.scan.p);
    entry_scan_emit_kernel<<<e.first[3], kScanThreads, 0, s>>>(e, R.scan.p);
    note_launch(2);
  } else {
    // chunk_len of every FO entry within its own diff
    if (nfo) MTC_CUDA_R(grid_scan(FoLen{R.fo_node.p, M, tree ? 1 : 0}, StoreExcl{R.fo_excl.p}, nullptr, nfo,
                                  R.scan.p, R.scan_total.p, s));
    // items of the main shift regions and of the chain's repeat maps
    if (nsh) MTC_CUDA_R(grid_scan(ShiftItems{a}, StoreShiftExcl{a}, nullptr, nsh, R.scan.p, R.tot.p + 4, s));
    if (nfo_chain) {
      chain_ranges_kernel<<<gsz(nfo_chain), 256, 0, s>>>(a, nfo_chain);
      note_launch();
      MTC_CUDA_R(grid_scan(ChainDmCount{a}, StoreExcl{R.dm_excl.p}, nullptr, nfo_chain, R.scan.p, R.tot.p + 0, s));
    }
  }
  // chunk_len relative to each FO entry's own diff; the main checkpoint's FO
  // items (tot[2])
  if (nfo) {
    clen_kernel<<<gsz(nfo), 256, 0, s>>>(a);
    note_launch();
  }
  // chain tables on the second stream, after the clears and the entries
  MTC_CUDA_R(cudaEventRecord(rev_[2], s));
  if (nsteps) {
    MTC_CUDA_R(cudaStreamWaitEvent(side, rev_[2], 0));
    chain_tables_kernel<<<num_sms() * 8, 256, 0, side>>>(a);
    note_launch();
  }
  MTC_CUDA_R(cudaEventRecord(rev_[3], side));
  // main checkpoint, beside them
  MTC_CUDA_R(cudaStreamWaitEvent(s, rev_[1], 0));
  if (di[0].F) { fo_at_kernel<<<gsz(di[0].F), 256, 0, s>>>(a); note_launch(); }
  if (di[0].S) {
    main_shift_kernel<<<gsz(di[0].S), 256, 0, s>>>(a);
    note_launch();
  }
  if (di[0].F || di[0].S) {
    main_cover_kernel<<<num_sms() * 8, 256, 0, s>>>(a);
    note_launch();
  }
  MTC_CUDA_R(cudaStreamWaitEvent(s, rev_[3], 0));
  // 4: every chunk's source, 5: the copy; range by range, each range copied
  // on the second stream while the next is resolved
  StepTimer t_rc("restart: resolve and copy launches", N);
  const uint32_t parts = restart_parts(N);
  const uint64_t per = ((uint64_t)N + parts - 1) / parts;
  const uint64_t step = (per + 31) / 32 * 32;
  uint32_t launched = 0;
  for (uint64_t lo = 0; lo < N; lo += step, launched++) {
    RArgs r = a;
    r.c_lo = (uint32_t)lo;
    r.c_hi = (uint32_t)std::min<uint64_t>(N, lo + step);
    resolve_kernel<<<std::min(gsz(r.c_hi - r.c_lo), resolve_grid()), 256, 0, s>>>(r);
    if (parts == 1) {
      restore_copy_kernel<<<num_sms() * 3, 256, 0, s>>>(r);
    } else {
      MTC_CUDA_R(cudaEventRecord(rev_[4 + launched], s));
      MTC_CUDA_R(cudaStreamWaitEvent(side, rev_[4 + launched], 0));
      restore_copy_kernel<<<num_sms() * 3, 256, 0, side>>>(r);
    }
    note_launch(2);
  }
  if (parts > 1) {
    MTC_CUDA_R(cudaEventRecord(rev_[11], side));
    MTC_CUDA_R(cudaStreamWaitEvent(s, rev_[11], 0));
  }
  cudaEventRecord(e1, s);
  Readback rb{};
  rb.src[0] = err_.p;
  rb.dst[0] = static_cast<uint32_t*>(host_alias(err_host_));
  rb.words[0] = 1;
  MTC_CUDA_R(launch_readback(rb, s));
  return ST_OK;
}

}  // namespace mtc
