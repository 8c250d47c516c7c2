// leaf_kernels.cu -- chunk hashing and per-chunk classification.
//
// One thread owns one chunk (Murmur3 and MD5 are serial over a chunk).  On the
// fast path the chunk bytes reach shared memory through TMA tiled loads: the
// buffer is viewed as a 2-D tensor [n_full rows x cs bytes]; each stage moves a
// box of 256 rows x W bytes (W = 128, 64, 32 or 16) with the matching TMA
// swizzle so that the 256 consumer threads read their rows without bank
// conflicts.  A dedicated producer warp keeps STAGES boxes in flight; full/empty
// mbarriers hand stages between producer and consumers.  Odd chunk sizes,
// unaligned buffers and the partial last chunk use a thread-per-chunk kernel
// that reads global memory directly.  Both end in the same epilogue, which
// restates the leaf loops of the reference:
//   tree  -- src/tree_approach.cpp:57-94 (baseline) and :309-351
//   list  -- src/list_approach.cpp:38-61
//   basic -- src/basic_approach.cpp:25-46
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <utility>

#include "mtc_common.cuh"
#include "mtc_internal.hpp"
#include "mtc_tma.cuh"

namespace mtc {

namespace {
// R (template) = consumer threads = chunks per tile = TMA box rows; one
// producer warp more per CTA
constexpr int kStages = 3;    // boxes in flight per CTA

template <int W>
__device__ __forceinline__ uint32_t swz(uint32_t logical) {
  constexpr uint32_t mask = W == 128 ? 7u : W == 64 ? 3u : W == 32 ? 1u : 0u;
  return logical ^ (((logical >> 7) & mask) << 4);
}

constexpr uint8_t PENDING = 0xFE;  // changed chunk, classified by the insert pass

// Append chunk c to the changed list (one atomic per warp).
// Appends a changed chunk to the list the map inserts read (warp-aggregated).
__device__ __forceinline__ void append_changed(const LeafArgs& a, bool changed, uint32_t c) {
  const unsigned act = __activemask();
  const unsigned b = __ballot_sync(act, changed);
  if (!b) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(b) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(a.changed_count, (uint32_t)__popc(b));
  base = __shfl_sync(act, base, leader);
  if (changed) a.changed_list[base + __popc(b & ((1u << lane) - 1))] = c;
}

// Streaming part of the per-chunk work: compare with the previous digest,
// store the new one.  Map inserts happen in leaf_insert_kernel so that the
// hashing pipeline never waits on random memory accesses.
template <int EPI>
__device__ __forceinline__ void leaf_epilogue(const LeafArgs& a, bool valid, uint32_t c, const Digest& dg,
                                              const Digest& old) {
  if (EPI == EPI_HASH) {
    if (valid) st_digest(a.out + c, dg);
    return;
  }
  if (EPI == EPI_BASIC) {
    if (!valid) return;
    uint8_t changed = 1;
    if (!a.basic_first && digest_eq(dg, old)) changed = 0;
    if (changed) st_digest(a.prev + c, dg);
    a.labels[c] = changed;
    return;
  }
  // tree (src/tree_approach.cpp:326-349) and list (src/list_approach.cpp:50-59)
  bool changed = false;
  if (valid) {
    changed = !digest_eq(dg, old);
    if (changed) st_digest(a.prev + c, dg);
    a.labels[c] = changed ? PENDING : (EPI == EPI_TREE ? FIXED_DUPL : DONE);
    // A FIXED_DUPL leaf's insert() always finds its digest (every earlier
    // leaf digest was inserted) and changes nothing, so it is not repeated.
  }
  append_changed(a, changed, c);
}

// A note for the demote pass (a changed-list position); kCheckCreator: the
// chunk met an entry that another insert of this launch created, whose chunk
// is checked too.
constexpr uint32_t kCheckCreator = 1u << 31;  // chunk counts stay below 2^31
// Every changed chunk notes itself at most once, so the notes never outnumber
// the changed chunks (the list holds N + 1 entries).
__device__ __forceinline__ void note_dup(const LeafArgs& a, uint32_t note) {
  const uint32_t k = atomicAdd(a.dup_count, 1u);
  if (k < a.dup_cap) a.dup_list[k] = note;
  else raise_err(a.err, DERR_CAPACITY);
}

// Map insert of one changed chunk (src/tree_approach.cpp:325-349,
// src/list_approach.cpp:50-59): new digest -> first occurrence; a digest
// already inserted by this launch -> first occurrence for now, the lowest
// chunk keeping the entry; an older digest -> shifted duplicate, except (tree)
// one whose entry carries this checkpoint's id, which an id that was not
// advanced (the header overload) leaves in place: the reference lowers its
// node and keeps the chunk a first occurrence there too.  The creator of an
// entry waits for nothing after its claim.
template <int EPI>
__global__ void leaf_insert_kernel(LeafArgs a) {
  pdl_enter();
  const uint32_t n = *a.changed_count;
  const uint32_t cur = a.sp->cur, epoch = a.sp->epoch;
  uint32_t created = 0;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t c = a.changed_list[k];
    const Digest dg = map_key(ld_digest(a.prev + c));
    const uint32_t node = EPI == EPI_TREE ? a.leaf_base + c : c;
    uint64_t slot = 0;
    uint8_t label = SHIFT_DUPL;
    const int r = map_claim(a.map, dg, &slot, a.err);
    MapSlot* s = &a.map.slots[slot];
    if (r == INS_NEW) {
      s->tree = cur;
      s->first_chunk = c;
      atomicMin(&s->win, win_of(epoch, node));
      label = FIRST_OCUR;
      created++;
    } else if (r == INS_EXISTING) {
      const unsigned long long old = win_min(&s->win, win_of(epoch, node));
      if (old == kWinEmpty || win_epoch(old) == epoch) {
        label = FIRST_OCUR;  // first seen by this launch: the lowest chunk keeps it
        note_dup(a, (uint32_t)k | kCheckCreator);
      } else if (EPI == EPI_TREE && __ldcg(&s->tree) == cur) {
        // lowest node within the older entry (the reference's atomic_min,
        // src/tree_approach.cpp:337-339): the entry's high bits (epoch and
        // serial level) are fixed, since every insert of this launch carries
        // a larger epoch and leaves them alone, so one atomicMin on the
        // whole word lowers exactly its node
        if (win_node(old) > node) win_min(&s->win, (old & ~0xffffffffull) | node);
        label = FIRST_OCUR;
        note_dup(a, (uint32_t)k);
      }
    }
    a.chunk_slot[k] = (uint32_t)slot;  // by list position: a sequential write
    a.labels[c] = label;
  }
  count_new_entries(a.map, created);
}

// Second pass (src/tree_approach.cpp:356-369): a first occurrence that does
// not own its digest becomes a shifted duplicate.  Only the noted chunks and
// the creators of their entries can be such.
__device__ __forceinline__ void demote_chunk(const LeafArgs& a, uint32_t c, const MapSlot* s, uint32_t cur) {
  if (a.labels[c] != FIRST_OCUR) return;
  const uint32_t node = a.leaf_base + c;
  const uint32_t owner = win_node(s->win);
  if (a.epi == EPI_TREE ? (s->tree == cur && owner != node) : (owner != node)) {
    a.labels[c] = SHIFT_DUPL;
    if (a.demoted) atomicOr(a.demoted, 1u);
  }
}
__global__ void leaf_demote_kernel(LeafArgs a) {
  pdl_enter();
  const uint32_t n = min(*a.dup_count, a.dup_cap);
  const uint32_t cur = a.sp->cur;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t e = a.dup_list[i];
    const uint32_t k = e & ~kCheckCreator;
    const uint32_t c = a.changed_list[k];
    const MapSlot* s = &a.map.slots[a.chunk_slot[k]];
    demote_chunk(a, c, s, cur);
    if (e & kCheckCreator) demote_chunk(a, s->first_chunk, s, cur);
  }
}

template <int EPI>
__device__ __forceinline__ bool needs_old(const LeafArgs& a) {
  return EPI != EPI_HASH && !(EPI == EPI_BASIC && a.basic_first);
}

// ---------------------------------------------------------------------------
// TMA pipeline kernel.
// ---------------------------------------------------------------------------
template <int HK, int EPI, int W, int kRows>
__global__ void __launch_bounds__(kRows + 32, 2) leaf_tma_kernel(const __grid_constant__ CUtensorMap tmap, LeafArgs a,
                                                              uint32_t n_full) {
  pdl_enter();
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr uint32_t kStageBytes = kRows * W;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  const int tid = threadIdx.x;
  const uint32_t xsteps = a.cs / W;
  const uint32_t ntiles = (n_full + kRows - 1) / kRows;
  const uint32_t limit = a.spin_limit ? a.spin_limit : kMbarSpinLimit;

  if (tid == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kRows / 32);
    }
    mbar_fence_init();
  }
  __syncthreads();

  if (tid >= kRows) {
    // producer warp: one elected lane issues every box in consumption order
    if (tid == kRows) {
      tma_prefetch_desc(&tmap);
      uint32_t it = 0;
      bool ok = !a.stall;  // injected fault: no copy is ever issued
      for (uint32_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        for (uint32_t xs = 0; xs < xsteps; xs++, it++) {
          const uint32_t s = it % kStages, ph = (it / kStages) & 1;
          if (!mbar_wait(&empty[s], ph ^ 1, limit)) { raise_err(a.err, DERR_SPIN); ok = false; break; }
          mbar_arrive_expect_tx(&full[s], kStageBytes);
          tma_load_2d(smem + s * kStageBytes, &tmap, (int32_t)(xs * W), (int32_t)(tile * kRows), &full[s]);
        }
      }
      // drain: every issued box must land before the CTA may exit
      uint32_t first = it > (uint32_t)kStages ? it - kStages : 0;
      for (uint32_t j = first; j < it; j++) mbar_wait(&full[j % kStages], (j / kStages) & 1);
    }
    return;
  }

  const uint32_t lane = tid & 31;
  uint32_t it = 0;
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint32_t c = tile * kRows + tid;
    const bool valid = c < n_full;
    Digest old{{0, 0, 0, 0}};
    if (valid && needs_old<EPI>(a)) old = ld_digest(a.prev + c);
    Murmur3State mm;
    Md5State md;
    if (HK == HASH_MD5) md.init(); else mm.init();
    uint32_t X[16];
    for (uint32_t xs = 0; xs < xsteps; xs++, it++) {
      const uint32_t s = it % kStages, ph = (it / kStages) & 1;
      if (!mbar_wait(&full[s], ph, limit)) { raise_err(a.err, DERR_SPIN); return; }
      const uint8_t* stage = smem + s * kStageBytes;
      const uint32_t rowbase = (uint32_t)tid * W;
      // the row into registers, then the stage goes back to the producer
      // before any hashing: the refill overlaps this thread's hash work
      uint4 row[W / 16];
#pragma unroll
      for (int q = 0; q < W / 16; q++) row[q] = *reinterpret_cast<const uint4*>(stage + swz<W>(rowbase + q * 16));
      // release the stage: this thread's reads before the refill's TMA write
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (HK == HASH_MD5) {
        if (W >= 64) {
#pragma unroll
          for (int blk = 0; blk < W / 64; blk++) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const uint4 v = row[blk * 4 + q];
              X[4 * q] = v.x; X[4 * q + 1] = v.y; X[4 * q + 2] = v.z; X[4 * q + 3] = v.w;
            }
            md.block(X);
          }
        } else {
#pragma unroll
          for (int i = 0; i < 16; i++) X[i] = 0;
#pragma unroll
          for (int q = 0; q < W / 16; q++) {
            const uint4 v = row[q];
            X[4 * q] = v.x; X[4 * q + 1] = v.y; X[4 * q + 2] = v.z; X[4 * q + 3] = v.w;
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < W / 16; q++) mm.block(row[q].x, row[q].y, row[q].z, row[q].w);
      }
    }
    Digest dg;
    if (HK == HASH_MD5) {
      if (W >= 64) {
#pragma unroll
        for (int i = 0; i < 16; i++) X[i] = 0;
        dg = md.finish(X, 0, a.cs);
      } else {
        dg = md.finish(X, a.cs, a.cs);
      }
    } else {
      dg = mm.finish(a.cs);
    }
    leaf_epilogue<EPI>(a, valid, c, dg, old);
  }
}

// ---------------------------------------------------------------------------
// Thread-per-chunk kernel reading global memory directly, for chunks
// [c0, c1).
// ---------------------------------------------------------------------------
template <int EPI>
__global__ void leaf_direct_kernel(LeafArgs a, uint32_t c0, uint32_t c1) {
  pdl_enter();
  for (uint64_t c = c0 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < c1; c += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t off = c * (uint64_t)a.cs;
    uint64_t nb = a.cs;
    if (c == a.n_chunks - 1) nb = a.len - off;
    Digest old{{0, 0, 0, 0}};
    if (needs_old<EPI>(a)) old = ld_digest(a.prev + c);
    Digest dg = hash_bytes(a.hash_kind, a.data + off, nb);
    leaf_epilogue<EPI>(a, true, (uint32_t)c, dg, old);
  }
}

// ---------------------------------------------------------------------------
// One persistent launch for the leaf pass of many deduplicators (a batch).
// A device work queue holds (member, tile) items; each CTA's producer lane
// claims the next item with one atomicAdd and streams its boxes through the
// same full/empty mbarrier pipeline as leaf_tma_kernel, announcing in a small
// per-stage record which member, tile and column step each box belongs to.
// Members differ in chunk size (box width 64 or 128 bytes), digest and
// approach; every consumer thread owns one row of the current item and ends
// with that member's epilogue.  Items are ordered largest first.  A producer
// that finds the queue empty drains its copies, then sends one record
// without data that stops the CTA's consumers.
// ---------------------------------------------------------------------------
struct BatchStageMeta {
  uint32_t member, tile, xs, flags;  // flags: kMetaFirst | kMetaLast | kMetaDone
};
constexpr uint32_t kMetaFirst = 1, kMetaLast = 2, kMetaDone = 4;
constexpr uint32_t kBatchStageBytes = kBatchRows * 128;

__device__ __forceinline__ bool needs_old_rt(const LeafArgs& a) {
  return a.epi != EPI_HASH && !(a.epi == EPI_BASIC && a.basic_first);
}

__global__ void __launch_bounds__(kBatchRows + 32, 3) batch_leaf_kernel(BatchLeafParams p) {
  pdl_enter();
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * kBatchStageBytes);
  uint64_t* empty = full + kStages;
  BatchStageMeta* meta = reinterpret_cast<BatchStageMeta*>(empty + kStages);
  const int tid = threadIdx.x;
  const uint32_t limit = p.spin_limit ? p.spin_limit : kMbarSpinLimit;
  if (tid == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kBatchRows / 32);
    }
    mbar_fence_init();
  }
  __syncthreads();

  if (tid >= kBatchRows) {
    if (tid == kBatchRows) {
      uint32_t it = 0;
      uint32_t* err = p.members[0].la.err;
      bool ok = true;
      while (ok) {
        const uint32_t k = atomicAdd(p.head, 1u);
        if (k >= p.nitems) break;
        const uint2 item = p.items[k];
        const uint32_t m = item.x, tile = item.y;
        const uint32_t xsteps = p.members[m].xsteps, W = p.members[m].W;
        err = p.members[m].la.err;
        for (uint32_t xs = 0; xs < xsteps; xs++, it++) {
          const uint32_t s = it % kStages, ph = (it / kStages) & 1;
          if (!mbar_wait(&empty[s], ph ^ 1, limit)) {
            raise_err(err, DERR_SPIN);
            ok = false;
            break;
          }
          meta[s] = BatchStageMeta{m, tile, xs, (xs == 0 ? kMetaFirst : 0u) | (xs + 1 == xsteps ? kMetaLast : 0u)};
          mbar_arrive_expect_tx(&full[s], kBatchRows * W);
          tma_load_2d(smem + s * kBatchStageBytes, &p.members[m].map, (int32_t)(xs * W), (int32_t)(tile * kBatchRows),
                      &full[s]);
        }
      }
      // drain: every issued box lands before the CTA exits (before the stop
      // record, which reuses the slot of the oldest of them)
      const uint32_t first = it > (uint32_t)kStages ? it - kStages : 0;
      for (uint32_t j2 = first; j2 < it; j2++) mbar_wait(&full[j2 % kStages], (j2 / kStages) & 1, limit);
      if (ok) {
        // the stop record: no data, the arrive alone completes the phase
        const uint32_t s = it % kStages, ph = (it / kStages) & 1;
        if (mbar_wait(&empty[s], ph ^ 1, limit)) {
          meta[s] = BatchStageMeta{0, 0, 0, kMetaDone};
          mbar_arrive(&full[s]);
        } else {
          raise_err(err, DERR_SPIN);
        }
      }
    }
    return;
  }

  const uint32_t lane = tid & 31;
  Murmur3State mm;
  Md5State md;
  mm.init();
  md.init();
  Digest old{{0, 0, 0, 0}};
  uint32_t c = 0;
  bool valid = false;
  for (uint32_t it = 0;; it++) {
    const uint32_t s = it % kStages, ph = (it / kStages) & 1;
    if (!mbar_wait(&full[s], ph, limit)) {
      raise_err(p.members[0].la.err, DERR_SPIN);
      return;
    }
    const BatchStageMeta mt = meta[s];
    if (mt.flags & kMetaDone) return;
    const MemberLeaf& ml = p.members[mt.member];
    const LeafArgs& a = ml.la;
    const uint32_t W = ml.W;
    const bool md5 = a.hash_kind == HASH_MD5;
    if (mt.flags & kMetaFirst) {
      c = mt.tile * kBatchRows + tid;
      valid = c < ml.n_full;
      old = Digest{{0, 0, 0, 0}};
      if (valid && needs_old_rt(a)) old = ld_digest(a.prev + c);
      mm.init();
      md.init();
    }
    // the row into registers, then the stage goes back to the producer
    const uint8_t* stage = smem + s * kBatchStageBytes;
    uint4 row[8];
    if (W == 128) {
#pragma unroll
      for (int q = 0; q < 8; q++) row[q] = *reinterpret_cast<const uint4*>(stage + swz<128>((uint32_t)tid * 128 + q * 16));
    } else {
#pragma unroll
      for (int q = 0; q < 4; q++) row[q] = *reinterpret_cast<const uint4*>(stage + swz<64>((uint32_t)tid * 64 + q * 16));
    }
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
    const int nblk = W == 128 ? 2 : 1;
    if (md5) {
      uint32_t X[16];
      for (int blk = 0; blk < nblk; blk++) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const uint4 v = row[blk * 4 + q];
          X[4 * q] = v.x; X[4 * q + 1] = v.y; X[4 * q + 2] = v.z; X[4 * q + 3] = v.w;
        }
        md.block(X);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (q < 4 * nblk) mm.block(row[q].x, row[q].y, row[q].z, row[q].w);
    }
    if (mt.flags & kMetaLast) {
      Digest dg;
      if (md5) {
        uint32_t X[16];
#pragma unroll
        for (int i = 0; i < 16; i++) X[i] = 0;
        dg = md.finish(X, 0, a.cs);
      } else {
        dg = mm.finish(a.cs);
      }
      switch (a.epi) {
        case EPI_TREE: leaf_epilogue<EPI_TREE>(a, valid, c, dg, old); break;
        case EPI_LIST: leaf_epilogue<EPI_LIST>(a, valid, c, dg, old); break;
        case EPI_BASIC: leaf_epilogue<EPI_BASIC>(a, valid, c, dg, old); break;
        default: leaf_epilogue<EPI_HASH>(a, valid, c, dg, old); break;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Warp-per-chunk kernel: the lanes of a warp load one chunk together into
// shared memory (coalesced 4-byte words), then lane 0 hashes it.  The digests
// are serial chains (each 16-byte Murmur3 block and each 64-byte MD5 block
// depends on the state left by the previous one), so the other lanes cannot
// share the hashing; this shape exists for the autotuner to compare against
// the thread-per-chunk pipelines.
// ---------------------------------------------------------------------------
constexpr uint32_t kWarpChunkMax = 4096;
template <int EPI>
__global__ void leaf_warp_kernel(LeafArgs a, uint32_t c0, uint32_t c1) {
  pdl_enter();
  extern __shared__ uint32_t wsm[];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t stride_w = (a.cs + 64 + 3) / 4;  // words per warp buffer, zero padding included
  uint32_t* buf = wsm + warp * stride_w;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const bool al4 = (reinterpret_cast<uintptr_t>(a.data) & 3) == 0 && (a.cs & 3) == 0;
  for (uint64_t c = c0 + (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); c < c1; c += nwarps) {
    const uint64_t off = c * (uint64_t)a.cs;
    const uint32_t nb = c == a.n_chunks - 1 ? (uint32_t)(a.len - off) : a.cs;
    const uint32_t nw = (nb + 64 + 3) / 4;
    for (uint32_t i = lane; i < nw; i += 32) {
      uint32_t v = 0;
      if (al4 && 4 * i + 4 <= nb) v = __ldg(reinterpret_cast<const uint32_t*>(a.data + off) + i);
      else v = ld_word_any(a.data + off, 4 * (uint64_t)i, nb);
      buf[i] = v;
    }
    __syncwarp();
    if (lane == 0) {
      Digest old{{0, 0, 0, 0}};
      if (needs_old<EPI>(a)) old = ld_digest(a.prev + c);
      const Digest dg = hash_words(a.hash_kind, buf, nb);
      leaf_epilogue<EPI>(a, true, (uint32_t)c, dg, old);
    }
    __syncwarp();
  }
}

template <int EPI>
cudaError_t launch_warp(const LeafArgs& a, uint32_t c0, uint32_t c1, cudaStream_t s) {
  if (c1 <= c0) return cudaSuccess;
  const uint32_t warps_per_block = 8;
  const size_t smem = (size_t)warps_per_block * 4 * ((a.cs + 64 + 3) / 4);
  static std::atomic<bool> attr_set{false};
  if (!attr_set.load(std::memory_order_acquire)) {
    cudaError_t e = cudaFuncSetAttribute(leaf_warp_kernel<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(warps_per_block * 4 * ((kWarpChunkMax + 64 + 3) / 4)));
    if (e != cudaSuccess) return e;
    attr_set.store(true, std::memory_order_release);
  }
  uint64_t grid = (c1 - c0 + warps_per_block - 1) / warps_per_block;
  const uint64_t cap = (uint64_t)num_sms() * 8;
  if (grid > cap) grid = cap;
  static const bool reg =
      (register_input_kernel(reinterpret_cast<const void*>(leaf_warp_kernel<EPI>), INPUT_LEAF_DIRECT), true);
  (void)reg;
  launch_k(leaf_warp_kernel<EPI>, (uint32_t)grid, warps_per_block * 32, smem, s, a, c0, c1);
  note_launch();
  return cudaGetLastError();
}

cudaError_t dispatch_warp(const LeafArgs& a, uint32_t c0, uint32_t c1, cudaStream_t s) {
  switch (a.epi) {
    case EPI_TREE: return launch_warp<EPI_TREE>(a, c0, c1, s);
    case EPI_LIST: return launch_warp<EPI_LIST>(a, c0, c1, s);
    case EPI_BASIC: return launch_warp<EPI_BASIC>(a, c0, c1, s);
    default: return launch_warp<EPI_HASH>(a, c0, c1, s);
  }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

int tma_width(uint32_t cs) {
  if (cs % 128 == 0) return 128;
  if (cs == 64 || cs == 32 || cs == 16) return (int)cs;
  return 0;
}

bool make_tmap(TmaCache* c, const uint8_t* data, uint64_t len, uint32_t cs, int W, int rows, uint32_t n_full) {
  if (c->ptr == data && c->len == len && c->cs == cs && c->width == W && c->rows == rows) return true;
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {cs, n_full};
  cuuint64_t strides[1] = {cs};
  cuuint32_t box[2] = {(cuuint32_t)W, (cuuint32_t)rows};
  cuuint32_t estr[2] = {1, 1};
  CUtensorMapSwizzle sw = W == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                        : W == 64  ? CU_TENSOR_MAP_SWIZZLE_64B
                        : W == 32  ? CU_TENSOR_MAP_SWIZZLE_32B
                                   : CU_TENSOR_MAP_SWIZZLE_NONE;
  CUresult r = fn(&c->map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<uint8_t*>(data), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) { c->ptr = nullptr; return false; }
  c->ptr = data; c->len = len; c->cs = cs; c->width = W; c->rows = rows;
  return true;
}

template <int HK, int EPI, int W, int R>
cudaError_t launch_tma_t(const LeafArgs& a, const CUtensorMap& m, uint32_t n_full, int ctas_per_sm, cudaStream_t s) {
  auto k = leaf_tma_kernel<HK, EPI, W, R>;
  static const bool reg = (register_input_kernel(reinterpret_cast<const void*>(k), INPUT_LEAF_TMA), true);
  (void)reg;
  const size_t smem = 1024 + (size_t)kStages * R * W + 2 * kStages * sizeof(uint64_t);
  static std::atomic<bool> attr_set{false};
  if (!attr_set.load(std::memory_order_acquire)) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set.store(true, std::memory_order_release);
  }
  const uint32_t ntiles = (n_full + R - 1) / R;
  // resident CTAs per SM that fit in 227 KB of shared memory, at most 3 by default
  const int fit = (int)((227u * 1024u) / smem);
  int per_sm = ctas_per_sm > 0 ? ctas_per_sm : 3;
  if (per_sm > fit) per_sm = fit > 0 ? fit : 1;
  uint32_t grid = (uint32_t)(num_sms() * per_sm);
  if (grid > ntiles) grid = ntiles;
  launch_k(k, grid, R + 32, smem, s, m, a, n_full);
  note_launch();
  return cudaGetLastError();
}

template <int HK, int EPI, int R>
cudaError_t launch_tma_w(const LeafArgs& a, const CUtensorMap& m, uint32_t n_full, int W, int per_sm, cudaStream_t s) {
  switch (W) {
    case 128: return launch_tma_t<HK, EPI, 128, R>(a, m, n_full, per_sm, s);
    case 64: return launch_tma_t<HK, EPI, 64, R>(a, m, n_full, per_sm, s);
    case 32: return launch_tma_t<HK, EPI, 32, R>(a, m, n_full, per_sm, s);
    default: return launch_tma_t<HK, EPI, 16, R>(a, m, n_full, per_sm, s);
  }
}

template <int EPI>
cudaError_t launch_tma_e(const LeafArgs& a, const CUtensorMap& m, uint32_t n_full, int W, const LeafTune& t,
                         cudaStream_t s) {
  if (t.rows == 128) {
    if (a.hash_kind == HASH_MD5) return launch_tma_w<HASH_MD5, EPI, 128>(a, m, n_full, W, t.ctas_per_sm, s);
    return launch_tma_w<HASH_MURMUR3, EPI, 128>(a, m, n_full, W, t.ctas_per_sm, s);
  }
  if (a.hash_kind == HASH_MD5) return launch_tma_w<HASH_MD5, EPI, 256>(a, m, n_full, W, t.ctas_per_sm, s);
  return launch_tma_w<HASH_MURMUR3, EPI, 256>(a, m, n_full, W, t.ctas_per_sm, s);
}

template <int EPI>
cudaError_t launch_direct(const LeafArgs& a, uint32_t c0, uint32_t c1, cudaStream_t s) {
  if (c1 <= c0) return cudaSuccess;
  uint64_t n = c1 - c0;
  uint32_t grid = (uint32_t)((n + 127) / 128);
  uint32_t cap = (uint32_t)num_sms() * 16;
  if (grid > cap) grid = cap;
  static const bool reg =
      (register_input_kernel(reinterpret_cast<const void*>(leaf_direct_kernel<EPI>), INPUT_LEAF_DIRECT), true);
  (void)reg;
  launch_k(leaf_direct_kernel<EPI>, grid, 128, 0, s, a, c0, c1);
  note_launch();
  return cudaGetLastError();
}

cudaError_t dispatch_direct(const LeafArgs& a, uint32_t c0, uint32_t c1, cudaStream_t s) {
  switch (a.epi) {
    case EPI_TREE: return launch_direct<EPI_TREE>(a, c0, c1, s);
    case EPI_LIST: return launch_direct<EPI_LIST>(a, c0, c1, s);
    case EPI_BASIC: return launch_direct<EPI_BASIC>(a, c0, c1, s);
    default: return launch_direct<EPI_HASH>(a, c0, c1, s);
  }
}
cudaError_t dispatch_tma(const LeafArgs& a, const CUtensorMap& m, uint32_t n_full, int W, const LeafTune& t,
                         cudaStream_t s) {
  switch (a.epi) {
    case EPI_TREE: return launch_tma_e<EPI_TREE>(a, m, n_full, W, t, s);
    case EPI_LIST: return launch_tma_e<EPI_LIST>(a, m, n_full, W, t, s);
    case EPI_BASIC: return launch_tma_e<EPI_BASIC>(a, m, n_full, W, t, s);
    default: return launch_tma_e<EPI_HASH>(a, m, n_full, W, t, s);
  }
}
}  // namespace

namespace {
// A fixed table (no heap allocation, so that launch sites reached from the
// allocation-free entry point allocate nothing either): one entry per kernel
// instantiation that reads the input, well below the capacity.
constexpr int kMaxInputKernels = 256;
std::mutex g_input_mu;
std::pair<const void*, int> g_input_kernels[kMaxInputKernels];
int g_input_count = 0;
}  // namespace
void register_input_kernel(const void* func, int kind) {
  std::lock_guard<std::mutex> lk(g_input_mu);
  if (g_input_count < kMaxInputKernels) g_input_kernels[g_input_count++] = {func, kind};
}
int input_kernel_kind(const void* func) {
  std::lock_guard<std::mutex> lk(g_input_mu);
  for (int i = 0; i < g_input_count; i++)
    if (g_input_kernels[i].first == func) return g_input_kernels[i].second;
  return INPUT_NONE;
}

namespace {
thread_local int t_pdl_suppress = 0;
}  // namespace
PdlSuppress::PdlSuppress() { t_pdl_suppress++; }
PdlSuppress::~PdlSuppress() { t_pdl_suppress--; }
bool pdl_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("MTCHECK_PDL");
    return !(e && e[0] == '0');
  }();
  return on && t_pdl_suppress == 0;
}

static std::atomic<uint64_t> g_launches{0};
void note_launch(uint32_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

bool input_tmap(TmaCache* c, const uint8_t* data, uint64_t len, uint32_t cs, const LeafTune& tune) {
  const uint32_t n_full = (uint32_t)(len / cs);
  const int W = tma_width(cs);
  const int rows = tune.rows != 128 ? 256 : 128;
  return W && n_full > 0 && (reinterpret_cast<uintptr_t>(data) & 15) == 0 &&
         make_tmap(c, data, len, cs, W, rows, n_full);
}

cudaError_t launch_leaves(const LeafArgs& a, TmaCache* cache, cudaStream_t s, const LeafTune& tune) {
  if (a.n_chunks == 0) return cudaSuccess;
  const uint32_t n_full = (uint32_t)(a.len / a.cs);
  const int W = tma_width(a.cs);
  const bool aligned = (reinterpret_cast<uintptr_t>(a.data) & 15) == 0;
  LeafTune t = tune;
  if (t.rows != 128) t.rows = 256;
  if (t.threads_per_chunk == 32 && a.cs <= kWarpChunkMax) return dispatch_warp(a, 0, a.n_chunks, s);
  uint32_t done = 0;
  if (!t.direct && W && aligned && n_full > 0 && cache && make_tmap(cache, a.data, a.len, a.cs, W, t.rows, n_full)) {
    cudaError_t e = dispatch_tma(a, cache->map, n_full, W, t, s);
    if (e != cudaSuccess) return e;
    done = n_full;
  }
  return dispatch_direct(a, done, a.n_chunks, s);
}

bool batch_leaf_member(MemberLeaf* out, const LeafArgs& a) {
  const int W = tma_width(a.cs);
  const uint32_t n_full = (uint32_t)(a.len / a.cs);
  if ((W != 64 && W != 128) || n_full == 0 || (reinterpret_cast<uintptr_t>(a.data) & 15) != 0) return false;
  TmaCache cache;
  if (!make_tmap(&cache, a.data, a.len, a.cs, W, kBatchRows, n_full)) return false;
  std::memcpy(&out->map, &cache.map, sizeof(CUtensorMap));
  out->la = a;
  out->n_full = n_full;
  out->W = (uint32_t)W;
  out->xsteps = a.cs / (uint32_t)W;
  out->pad = 0;
  return true;
}

cudaError_t launch_leaf_range(const LeafArgs& a, uint32_t c0, uint32_t c1, cudaStream_t s) {
  return dispatch_direct(a, c0, c1, s);
}

static size_t batch_leaf_smem() {
  return 1024 + (size_t)kStages * kBatchStageBytes + 2 * kStages * sizeof(uint64_t) + kStages * sizeof(BatchStageMeta);
}

cudaError_t batch_leaf_node_params(const BatchLeafParams& p, cudaKernelNodeParams* kp, void** args) {
  static std::atomic<bool> attr_set{false};
  const size_t smem = batch_leaf_smem();
  if (!attr_set.load(std::memory_order_acquire)) {
    cudaError_t e = cudaFuncSetAttribute(batch_leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set.store(true, std::memory_order_release);
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_leaf_kernel, kBatchRows + 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (per_sm > 3) per_sm = 3;
  uint32_t grid = (uint32_t)(num_sms() * per_sm);
  if (grid > p.nitems && p.nitems > 0) grid = p.nitems;
  args[0] = const_cast<BatchLeafParams*>(&p);
  kp->func = reinterpret_cast<void*>(batch_leaf_kernel);
  kp->gridDim = dim3(grid);
  kp->blockDim = dim3(kBatchRows + 32);
  kp->sharedMemBytes = (unsigned)smem;
  kp->kernelParams = args;
  kp->extra = nullptr;
  return cudaSuccess;
}

cudaError_t launch_leaf_inserts(const LeafArgs& a, cudaStream_t s) {
  const uint32_t grid = (uint32_t)num_sms() * 8;
  if (a.epi == EPI_TREE) launch_k(leaf_insert_kernel<EPI_TREE>, grid, 256, 0, s, a);
  else launch_k(leaf_insert_kernel<EPI_LIST>, grid, 256, 0, s, a);
  launch_k(leaf_demote_kernel, grid, 256, 0, s, a);
  note_launch(2);
  return cudaGetLastError();
}

}  // namespace mtc
