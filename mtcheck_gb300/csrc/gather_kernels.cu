// gather_kernels.cu -- everything between the leaf kernel and the finished
// incremental checkpoint in HBM:
//   * Merkle forest passes, one launch per tree level (src/tree_approach.cpp
//     :124-227 baseline, :378-477 incremental);
//   * deterministic compaction of region roots in the order a serial backend
//     pushes them (replaces the atomic Vector::push, include/kokkos_vector.hpp:37-40);
//   * diff assembly: region sizes, repeat-count table, stable sort of the
//     shifted duplicates by source checkpoint, metadata and the chunk gather
//     (src/tree_approach.cpp:512-710, src/list_approach.cpp:79-247,
//     src/basic_approach.cpp:52-143).
#include <cstdio>

#include "mtc_common.cuh"
#include "mtc_gather.hpp"
#include "mtc_scan.cuh"

namespace mtc {

namespace {

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
__global__ void fo_level_kernel(ForestArgs a, uint32_t beg, uint32_t end) {
  for (uint64_t n = beg + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n <= end; n += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t l = 2 * (uint32_t)n + 1, r = l + 1;
    if (a.labels[l] == FIRST_OCUR && a.labels[r] == FIRST_OCUR) {
      a.labels[n] = FIRST_OCUR;
      Digest d = hash_pair(a.hash_kind, ld_digest(a.tree + l), ld_digest(a.tree + r));
      st_digest(a.tree + n, d);
      map_insert_first(a.map, d, (uint32_t)n, a.cur, a.epoch, a.err);
    } else {
      a.labels[n] = DONE;
    }
  }
}

__device__ __forceinline__ uint8_t child_flag(uint8_t lab) {
  return (lab == FIXED_DUPL || lab == DONE) ? ROOT_NONE : (lab == SHIFT_DUPL ? ROOT_SHIFT : ROOT_FO);
}

// baseline != 0: the shift test reads the node's digest before it is hashed
// (src/tree_approach.cpp:202 vs :221).
__global__ void dup_level_kernel(ForestArgs a, uint32_t beg, uint32_t end, int baseline) {
  for (uint64_t n = beg + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n <= end; n += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t l = 2 * (uint32_t)n + 1, r = l + 1;
    const uint8_t ll = a.labels[l], lr = a.labels[r];
    uint8_t fl = ROOT_NONE, fr = ROOT_NONE;
    if (ll != lr) {
      a.labels[n] = DONE;
      fl = child_flag(ll);
      fr = child_flag(lr);
    } else if (ll == FIXED_DUPL) {
      a.labels[n] = FIXED_DUPL;
    } else if (ll == SHIFT_DUPL) {
      Digest d;
      if (baseline) {
        d = ld_digest(a.tree + n);
      } else {
        d = hash_pair(a.hash_kind, ld_digest(a.tree + l), ld_digest(a.tree + r));
        st_digest(a.tree + n, d);
      }
      if (map_find(a.map, d, a.err) >= 0) {
        a.labels[n] = SHIFT_DUPL;
      } else {
        a.labels[n] = DONE;
        fl = ROOT_SHIFT;
        fr = ROOT_SHIFT;
      }
    }
    a.rflag[l] = fl;
    a.rflag[r] = fr;
  }
}

// baseline only: hash and insert every interior node of the level (:218-224)
__global__ void insert_level_kernel(ForestArgs a, uint32_t beg, uint32_t end) {
  for (uint64_t n = beg + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n <= end; n += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t l = 2 * (uint32_t)n + 1, r = l + 1;
    Digest d = hash_pair(a.hash_kind, ld_digest(a.tree + l), ld_digest(a.tree + r));
    st_digest(a.tree + n, d);
    map_insert_first(a.map, d, (uint32_t)n, a.cur, a.epoch, a.err);
  }
}

// ---------------------------------------------------------------------------
// Root compaction in serial push order.
// ---------------------------------------------------------------------------
struct LevelTable {
  uint32_t nlev;
  uint32_t first_node[33];  // first node of each level in output order
  uint64_t first_pos[34];   // position of that level's first node
};

// canonical position -> node
struct PosToNode {
  LevelTable t;
  int ascending;  // 1: plain ascending node order (std::set of roots)
  __device__ __forceinline__ uint32_t operator()(uint64_t p) const {
    if (ascending) return (uint32_t)p + 1;
    uint32_t k = 0;
    while (k + 1 < t.nlev && p >= t.first_pos[k + 1]) k++;
    return t.first_node[k] + (uint32_t)(p - t.first_pos[k]);
  }
};

struct RootVal {
  PosToNode map;
  const uint8_t* rflag;
  __device__ __forceinline__ uint64_t operator()(uint64_t p) const {
    uint8_t f = rflag[map(p)];
    return (f == ROOT_FO ? 1ull : 0ull) | (f == ROOT_SHIFT ? (1ull << 32) : 0ull);
  }
};
struct RootEmit {
  PosToNode map;
  uint32_t* fo_list;
  uint32_t* sh_list;
  const Layout* lay;
  __device__ __forceinline__ void operator()(uint64_t p, uint64_t ex, uint64_t v) const {
    if (!v) return;
    uint32_t node = map(p);
    if (v & 1ull) fo_list[lay->root_fo + (uint32_t)ex] = node;
    if (v >> 32) sh_list[(uint32_t)(ex >> 32)] = node;
  }
};

__global__ void root_prologue_kernel(const uint8_t* labels, uint32_t N, int ascending, uint32_t* fo_list, Layout* lay) {
  // the incremental/baseline passes push the root only for N >= 2
  // (src/tree_approach.cpp:384-393); the serial reference inserts it whenever
  // it is a first occurrence (include/reference_impl.hpp:105-106)
  uint32_t root = (labels[0] == FIRST_OCUR && (ascending || N >= 2)) ? 1u : 0u;
  lay->root_fo = root;
  if (root) fo_list[0] = 0;
}
__global__ void root_epilogue_kernel(const uint64_t* total, Layout* lay) {
  lay->F = lay->root_fo + (uint32_t)(*total);
  lay->S = (uint32_t)(*total >> 32);
}

// ---------------------------------------------------------------------------
// Diff assembly
// ---------------------------------------------------------------------------
// First-occurrence roots: region size if the root owns its digest.
__global__ void fo_prep_kernel(GatherArgs g) {
  const uint32_t F = g.lay->F;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < F; i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t node = g.fo_list[i];
    uint64_t v = 0;
    if (g.approach == APPROACH_TREE) {
      NodeIdDev prev = slot_value(g.map, map_find(g.map, ld_digest(g.digests + node), g.err));
      if (prev.node == node && prev.tree == g.cur) v = (1ull << 32) | num_leaf_descendents(node, g.M);
    } else {
      v = (1ull << 32) | 1ull;  // list / basic: one chunk per entry
    }
    g.fo_val[i] = v;
  }
}
struct FoVal {
  const uint64_t* fo_val;
  __device__ __forceinline__ uint64_t operator()(uint64_t i) const { return fo_val[i]; }
};
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
__global__ void fo_totals_kernel(const uint64_t* total, Layout* lay) {
  lay->num_distinct = (uint32_t)(*total >> 32);
  lay->chunk_counter = (uint32_t)(*total);
}

// Shifted duplicates: (source checkpoint, source node) of each root.
__global__ void shift_prep_kernel(GatherArgs g) {
  const uint32_t S = g.lay->S;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < S; i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t node = g.sh_list[i];
    int64_t slot = map_find(g.map, ld_digest(g.digests + node), g.err);
    NodeIdDev prev = slot_value(g.map, slot);
    if (slot < 0 || prev.tree > g.cur) { atomicOr(g.err, DERR_MISSING); prev.tree = 0; prev.node = 0; }
    g.sh_key[i] = prev.tree;
    g.sh_prev[i] = prev.node;
    atomicAdd(&g.hist[prev.tree], 1u);
  }
}

// One block: repeat-count table, layout, header; bin representatives for the
// list approach's BinOp1D.
__global__ void layout_kernel(GatherArgs g) {
  __shared__ uint64_t sh[33];
  Layout* lay = g.lay;
  const uint32_t K = g.cur + 1;
  const uint32_t F = lay->F, S = lay->S, nd = lay->num_distinct;
  // P = number of source checkpoints that occur; max_key = largest of them
  __shared__ uint32_t smax;
  if (threadIdx.x == 0) smax = 0;
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
    h32[0] = g.baseline_id;
    h32[1] = g.cur;
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
  const uint32_t nbins = g.approach == APPROACH_TREE ? g.cur : S;
  const double range = (double)(g.approach == APPROACH_TREE ? g.cur : max_key);
  const double mul = (range <= (double)nbins) ? 1.0 : (double)nbins / range;
  for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) {
    int bk = (int)(mul * (double)k);
    uint32_t rep = k;
    while (rep > 0 && (int)(mul * (double)(rep - 1)) == bk) rep--;
    g.rep[k] = rep;
  }
}

// Stable counting sort of the shift entries by representative key.
// Tile t counts its keys; matrix[key * T + t] (key-major).
__global__ void sort_count_kernel(GatherArgs g, uint32_t T) {
  extern __shared__ uint32_t cnt[];
  const uint32_t K = g.cur + 1, S = g.lay->S;
  for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) {
    for (uint32_t k = threadIdx.x; k < K; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    const uint64_t b = (uint64_t)t * kSortTile;
    for (uint64_t i = b + threadIdx.x; i < b + kSortTile && i < S; i += blockDim.x) atomicAdd(&cnt[g.rep[g.sh_key[i]]], 1u);
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
// one warp per tile; entries are placed in tile order, 32 at a time
__global__ void sort_scatter_kernel(GatherArgs g, uint32_t T) {
  extern __shared__ uint32_t cur[];
  const uint32_t K = g.cur + 1, S = g.lay->S;
  const uint32_t lane = threadIdx.x;
  if (!g.lay->ok) return;
  uint8_t* pairs = g.stage + g.lay->pad + g.lay->pairs_off;
  for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) {
    const uint64_t b = (uint64_t)t * kSortTile;
    if (b >= S) break;
    for (uint32_t k = lane; k < K; k += 32) cur[k] = (uint32_t)g.sort_mat[(uint64_t)k * T + t];
    __syncwarp();
    for (uint64_t i0 = b; i0 < b + kSortTile && i0 < S; i0 += 32) {
      const uint64_t i = i0 + lane;
      const bool v = i < S && i < b + kSortTile;
      const uint32_t key = v ? g.rep[g.sh_key[i]] : 0xffffffffu;
      const uint32_t peers = __match_any_sync(0xffffffffu, key);
      const uint32_t rank = __popc(peers & ((1u << lane) - 1));
      const uint32_t leader = __ffs(peers) - 1;
      uint32_t base = 0;
      if (v) base = cur[key];
      __syncwarp();
      if (v) {
        const uint32_t pos = base + rank;
        uint32_t* e = reinterpret_cast<uint32_t*>(pairs + 8ull * pos);
        e[0] = g.sh_list[i];
        e[1] = g.sh_prev[i];
        if (lane == leader) cur[key] = base + __popc(peers);
      }
      __syncwarp();
    }
    __syncwarp();
  }
}

// Chunk gather into the data section.  Regions (reg_chunk, reg_slot, reg_len)
// are sorted by slot; every 16-byte unit of the data section is written once.
// Each block owns a contiguous range of units, so a thread locates its region
// once by binary search and then walks forward.
__global__ void copy_kernel(GatherArgs g) {
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
  uint64_t slot = u * 16 / cs;
  uint32_t lo = 0, hi = R - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (g.reg_slot[mid] <= slot) lo = mid; else hi = mid - 1;
  }
  uint32_t r = lo;
  for (; u < u1; u += blockDim.x) {
    slot = u * 16 / cs;
    while (r + 1 < R && g.reg_slot[r + 1] <= slot) r++;
    const uint64_t within = u * 16 - slot * cs;
    const uint64_t chunk = (uint64_t)g.reg_chunk[r] + (slot - g.reg_slot[r]);
    uint4 v = make_uint4(0, 0, 0, 0);
    if (chunk < last || (chunk == last && within + 16 <= tail_len)) {
      v = __ldcs(reinterpret_cast<const uint4*>(g.data + chunk * cs + within));
    } else if (chunk == last && within < tail_len) {
      uint32_t w[4] = {0, 0, 0, 0};
      for (uint32_t b = 0; b < 16 && within + b < tail_len; b++) w[b >> 2] |= (uint32_t)g.data[chunk * cs + within + b] << (8 * (b & 3));
      v = make_uint4(w[0], w[1], w[2], w[3]);
    }
    // chunks past the end of the buffer stay zero (the reference reads out of bounds there)
    __stcs(reinterpret_cast<uint4*>(dst + u * 16), v);
  }
}

// Byte-granular gather for chunk sizes that are not multiples of 16 or
// buffers that are not 16-byte aligned.
__global__ void copy_bytes_kernel(GatherArgs g) {
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
  lay->root_fo = 0;
  lay->F = (uint32_t)(*total);
  lay->S = (uint32_t)(*total >> 32);
}

__global__ void map_rehash_kernel(DigestMap from, uint64_t from_cap, DigestMap to, uint32_t* err) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < from_cap; i += (uint64_t)gridDim.x * blockDim.x) {
    const MapSlot& s = from.slots[i];
    if (s.state != 2) continue;
    Digest k{{s.key[0], s.key[1], s.key[2], s.key[3]}};
    uint64_t slot;
    map_insert(to, k, s.node, s.tree, s.epoch, &slot, err);
  }
}

}  // namespace

cudaError_t launch_map_rehash(const DigestMap& from, uint64_t from_cap, const DigestMap& to, uint32_t* err,
                              cudaStream_t s) {
  map_rehash_kernel<<<grid_for(from_cap, 256), 256, 0, s>>>(from, from_cap, to, err);
  note_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
cudaError_t launch_fo_level(const ForestArgs& a, uint32_t beg, uint32_t end, cudaStream_t s) {
  fo_level_kernel<<<grid_for(end - beg + 1, 256), 256, 0, s>>>(a, beg, end);
  note_launch();
  return cudaGetLastError();
}
cudaError_t launch_dup_level(const ForestArgs& a, uint32_t beg, uint32_t end, int baseline, cudaStream_t s) {
  dup_level_kernel<<<grid_for(end - beg + 1, 256), 256, 0, s>>>(a, beg, end, baseline);
  note_launch();
  return cudaGetLastError();
}
cudaError_t launch_insert_level(const ForestArgs& a, uint32_t beg, uint32_t end, cudaStream_t s) {
  insert_level_kernel<<<grid_for(end - beg + 1, 256), 256, 0, s>>>(a, beg, end);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_root_compaction(const uint8_t* labels, const uint8_t* rflag, uint32_t N, uint32_t M, int ascending,
                                   uint32_t* fo_list, uint32_t* sh_list, Layout* lay, uint64_t* scan_scratch,
                                   uint64_t* scan_total, cudaStream_t s) {
  PosToNode map{};
  map.ascending = ascending;
  if (!ascending) {
    // levels by depth, deepest first; depth d holds nodes [2^d - 1, 2^(d+1) - 2]
    uint32_t D = 0;
    while (((2ull << D) - 1) < M) D++;  // depth of node M-1
    uint32_t k = 0;
    uint64_t pos = 0;
    for (int d = (int)D; d >= 1; d--) {
      uint64_t lo = (1ull << d) - 1, hi = (2ull << d) - 2;
      if (hi > M - 1) hi = M - 1;
      if (lo > hi) continue;
      map.t.first_node[k] = (uint32_t)lo;
      map.t.first_pos[k] = pos;
      pos += hi - lo + 1;
      k++;
    }
    map.t.nlev = k;
    map.t.first_pos[k] = pos;
  }
  root_prologue_kernel<<<1, 1, 0, s>>>(labels, N, ascending, fo_list, lay);
  note_launch();
  cudaError_t e = grid_scan(RootVal{map, rflag}, RootEmit{map, fo_list, sh_list, lay}, nullptr, (uint64_t)M - 1,
                            scan_scratch, scan_total, s);
  if (e != cudaSuccess) return e;
  root_epilogue_kernel<<<1, 1, 0, s>>>(scan_total, lay);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_chunk_compaction(const uint8_t* labels, uint32_t n_chunks, int basic, uint32_t* fo_list,
                                    uint32_t* sh_list, Layout* lay, uint64_t* scan_scratch, uint64_t* scan_total,
                                    cudaStream_t s) {
  cudaError_t e = grid_scan(ChunkVal{labels, basic}, ChunkEmit{fo_list, sh_list}, nullptr, n_chunks, scan_scratch,
                            scan_total, s);
  if (e != cudaSuccess) return e;
  chunk_totals_kernel<<<1, 1, 0, s>>>(scan_total, lay);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_assemble(const GatherArgs& g, uint64_t max_entries, cudaStream_t s) {
  cudaError_t e;
  // the FO metadata is written while scanning, so the pad must be known first:
  // pad depends on F, P, S; P needs the histogram.  Order: shift prep
  // (histogram), FO prep + scan (region sizes), layout (pad, table, header),
  // FO emit (metadata + regions), sort, copy.
  cudaMemsetAsync(g.hist, 0, sizeof(uint32_t) * ((size_t)g.cur + 1), s);
  const uint32_t gs = grid_for(max_entries, 256);
  shift_prep_kernel<<<gs, 256, 0, s>>>(g);
  fo_prep_kernel<<<gs, 256, 0, s>>>(g);
  // region totals first (phase 1+2 of the scan), then layout, then emit
  uint32_t ntiles = (uint32_t)((max_entries + kScanTile - 1) / kScanTile);
  if (ntiles == 0) ntiles = 1;
  scan_tile_sums_kernel<<<ntiles, kScanThreads, 0, s>>>(FoVal{g.fo_val}, &g.lay->F, 0, g.scan_scratch);
  scan_tile_offsets_kernel<<<1, 1024, 0, s>>>(g.scan_scratch, ntiles, g.scan_total);
  fo_totals_kernel<<<1, 1, 0, s>>>(g.scan_total, g.lay);
  layout_kernel<<<1, 1024, 0, s>>>(g);
  scan_emit_kernel<<<ntiles, kScanThreads, 0, s>>>(FoVal{g.fo_val}, FoEmit{g}, &g.lay->F, 0, g.scan_scratch);
  note_launch(7);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (g.approach != APPROACH_BASIC) {
    const uint32_t K = g.cur + 1;
    const uint32_t T = (uint32_t)((max_entries + kSortTile - 1) / kSortTile) + 1;
    const size_t smem = sizeof(uint32_t) * (size_t)K;
    if (smem > 200 * 1024) return cudaErrorNotSupported;
    static size_t attr_cnt = 0, attr_sc = 0;
    if (smem > 48 * 1024 && smem > attr_cnt) {
      cudaFuncSetAttribute(sort_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr_cnt = smem;
    }
    if (smem > 48 * 1024 && smem > attr_sc) {
      cudaFuncSetAttribute(sort_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr_sc = smem;
    }
    sort_count_kernel<<<grid_for(T, 1, 16), 256, smem, s>>>(g, T);
    e = grid_scan(MatVal{g.sort_mat}, MatEmit{g.sort_mat}, nullptr, (uint64_t)K * T, g.scan_scratch2, g.scan_total2, s);
    if (e != cudaSuccess) return e;
    sort_scatter_kernel<<<grid_for(T, 1, 16), 32, smem, s>>>(g, T);
    note_launch(2);
  }
  const bool vec = (g.cs % 16 == 0) && ((reinterpret_cast<uintptr_t>(g.data) & 15) == 0);
  if (vec) copy_kernel<<<num_sms() * 8, 256, 0, s>>>(g);
  else copy_bytes_kernel<<<num_sms() * 8, 256, 0, s>>>(g);
  note_launch();
  return cudaGetLastError();
}

}  // namespace mtc
