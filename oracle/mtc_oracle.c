/*
 * mtc_oracle.c -- CPU restatement of the MTCheck deduplication path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file; only tests/, __graft_entry__.smoke() and the cpu_baseline
 * leg of bench.py use it, and only as the checker / the timed CPU reference.
 *
 * Every function restates the reference's algorithm in plain serial C, in the
 * iteration order of a Kokkos Serial execution space (that order defines the
 * canonical byte layout of the .incr_chkpt files, because the reference fills
 * its root lists with atomic pushes).  Citations are file:line in the
 * TauferLab/MTCheck sources.
 *
 * Pinning: the two digest functions are checked bit-for-bit against the
 * reference's own hash headers compiled on the host (oracle/_ref) and against
 * the golden vectors generated from them (tests/golden/hash_vectors.json); the
 * tree labelling is checked against the ten known-answer tests of
 * test/test_case_01..10.cpp (tests/golden/tree_kat.json); restart is checked
 * by round trips as in test/{tree,list,basic,full}_chkpt.cpp.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>

#define ORC_EXPORT __attribute__((visibility("default")))

enum { ORC_OK = 0, ORC_EINVAL = 1, ORC_ECORRUPT = 2, ORC_ENOMEM = 3, ORC_EINTERNAL = 6 };
/* DedupMode values, include/utils.hpp:39-49 */
enum { A_FULL = 1, A_BASIC = 2, A_LIST = 3, A_TREE = 4, A_TREE_REF = 5, A_TREE_LOW_OFFSET = 6 };
enum { H_MURMUR3 = 0, H_MD5 = 1 };
/* Label, include/utils.hpp:51-57 */
enum { FIRST_OCUR = 0, FIXED_DUPL = 1, SHIFT_DUPL = 2, FIRST_DUPL = 3, DONE = 4 };

typedef struct { uint8_t d[16]; } digest_t;
typedef struct { uint32_t node, tree; } nodeid_t;

/* header_t, include/utils.hpp:29-37 (32 bytes, little endian) */
typedef struct {
  uint32_t ref_id, chkpt_id;
  uint64_t datalen;
  uint32_t chunk_size, num_first_ocur, num_prior_chkpts, num_shift_dupl;
} header_t;

/* ------------------------------------------------------------------------ */
/* Murmur3 variant: include/kokkos_murmur3.hpp:213-292, hash() :431-437.     */
/* rotl64 returns uint32_t (:30-31), so every rotated value is truncated.    */
/* ------------------------------------------------------------------------ */
static inline uint64_t ld64(const uint8_t* p) {
  uint64_t v = 0;
  for (int i = 7; i >= 0; i--) v = (v << 8) | p[i];
  return v;
}
static inline uint32_t rotl64_u32(uint64_t x, int r) { return (uint32_t)((x << r) | (x >> (64 - r))); }
static inline uint64_t fmix64(uint64_t k) {
  k ^= k >> 33; k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33; return k;
}
static void murmur3_variant(const uint8_t* data, uint64_t len, uint8_t out[16]) {
  const uint64_t nblocks = len / 16;
  uint64_t h1 = 0, h2 = 0; /* seed 0 */
  const uint64_t c1 = 0x87c37b91114253d5ULL, c2 = 0x4cf5ad432745937fULL;
  for (uint64_t i = 0; i < nblocks; i++) {
    uint64_t k1 = ld64(data + 16 * i), k2 = ld64(data + 16 * i + 8);
    k1 *= c1; k1 = rotl64_u32(k1, 31); k1 *= c2; h1 ^= k1;
    h1 = rotl64_u32(h1, 27); h1 += h2; h1 = h1 * 5 + 0x52dce729;
    k2 *= c2; k2 = rotl64_u32(k2, 33); k2 *= c1; h2 ^= k2;
    h2 = rotl64_u32(h2, 31); h2 += h1; h2 = h2 * 5 + 0x38495ab5;
  }
  const uint8_t* tail = data + nblocks * 16;
  uint64_t k1 = 0, k2 = 0;
  unsigned rem = (unsigned)(len & 15);
  if (rem > 8) {
    for (unsigned b = rem; b > 8; b--) k2 ^= ((uint64_t)tail[b - 1]) << (8 * (b - 9));
    k2 *= c2; k2 = rotl64_u32(k2, 33); k2 *= c1; h2 ^= k2;
  }
  if (rem > 0) {
    unsigned top = rem > 8 ? 8 : rem;
    for (unsigned b = top; b > 0; b--) k1 ^= ((uint64_t)tail[b - 1]) << (8 * (b - 1));
    k1 *= c1; k1 = rotl64_u32(k1, 31); k1 *= c2; h1 ^= k1;
  }
  h1 ^= len; h2 ^= len;
  h1 += h2; h2 += h1;
  h1 = fmix64(h1); h2 = fmix64(h2);
  h1 += h2; h2 += h1;
  for (int i = 0; i < 8; i++) { out[i] = (uint8_t)(h1 >> (8 * i)); out[8 + i] = (uint8_t)(h2 >> (8 * i)); }
}

/* ------------------------------------------------------------------------ */
/* MD5: include/kokkos_md5.hpp:48-323 (RFC 1321; PolarSSL-style update and  */
/* finish).  For len > INT_MAX the reference feeds 128-byte pieces and       */
/* replaces the last one by len%128 bytes (:293-301); restated as is.        */
/* ------------------------------------------------------------------------ */
typedef struct { uint32_t total[2]; uint32_t state[4]; uint8_t buffer[64]; } md5_ctx;
static const uint32_t MD5_T[64] = {
  0xd76aa478,0xe8c7b756,0x242070db,0xc1bdceee,0xf57c0faf,0x4787c62a,0xa8304613,0xfd469501,
  0x698098d8,0x8b44f7af,0xffff5bb1,0x895cd7be,0x6b901122,0xfd987193,0xa679438e,0x49b40821,
  0xf61e2562,0xc040b340,0x265e5a51,0xe9b6c7aa,0xd62f105d,0x02441453,0xd8a1e681,0xe7d3fbc8,
  0x21e1cde6,0xc33707d6,0xf4d50d87,0x455a14ed,0xa9e3e905,0xfcefa3f8,0x676f02d9,0x8d2a4c8a,
  0xfffa3942,0x8771f681,0x6d9d6122,0xfde5380c,0xa4beea44,0x4bdecfa9,0xf6bb4b60,0xbebfbc70,
  0x289b7ec6,0xeaa127fa,0xd4ef3085,0x04881d05,0xd9d4d039,0xe6db99e5,0x1fa27cf8,0xc4ac5665,
  0xf4292244,0x432aff97,0xab9423a7,0xfc93a039,0x655b59c3,0x8f0ccc92,0xffeff47d,0x85845dd1,
  0x6fa87e4f,0xfe2ce6e0,0xa3014314,0x4e0811a1,0xf7537e82,0xbd3af235,0x2ad7d2bb,0xeb86d391};
static const uint8_t MD5_S[64] = {
  7,12,17,22,7,12,17,22,7,12,17,22,7,12,17,22, 5,9,14,20,5,9,14,20,5,9,14,20,5,9,14,20,
  4,11,16,23,4,11,16,23,4,11,16,23,4,11,16,23, 6,10,15,21,6,10,15,21,6,10,15,21,6,10,15,21};
static inline uint32_t rol32(uint32_t x, unsigned n) { return (x << n) | (x >> (32 - n)); }
static void md5_block(md5_ctx* c, const uint8_t* p) {
  uint32_t X[16];
  for (int i = 0; i < 16; i++) X[i] = (uint32_t)p[4*i] | ((uint32_t)p[4*i+1] << 8) | ((uint32_t)p[4*i+2] << 16) | ((uint32_t)p[4*i+3] << 24);
  uint32_t a = c->state[0], b = c->state[1], cc = c->state[2], d = c->state[3];
  for (int i = 0; i < 64; i++) {
    uint32_t f; int g;
    if (i < 16) { f = d ^ (b & (cc ^ d)); g = i; }
    else if (i < 32) { f = cc ^ (d & (b ^ cc)); g = (5 * i + 1) & 15; }
    else if (i < 48) { f = b ^ cc ^ d; g = (3 * i + 5) & 15; }
    else { f = cc ^ (b | ~d); g = (7 * i) & 15; }
    uint32_t t = d; d = cc; cc = b;
    b = b + rol32(a + f + X[g] + MD5_T[i], MD5_S[i]);
    a = t;
  }
  c->state[0] += a; c->state[1] += b; c->state[2] += cc; c->state[3] += d;
}
static void md5_update(md5_ctx* c, const uint8_t* in, int ilen) {
  if (ilen <= 0) return;
  uint32_t left = c->total[0] & 0x3F;
  int fill = 64 - (int)left;
  c->total[0] += (uint32_t)ilen;
  if (c->total[0] < (uint32_t)ilen) c->total[1]++;
  if (left && ilen >= fill) {
    memcpy(c->buffer + left, in, (size_t)fill);
    md5_block(c, c->buffer);
    in += fill; ilen -= fill; left = 0;
  }
  while (ilen >= 64) { md5_block(c, in); in += 64; ilen -= 64; }
  if (ilen > 0) memcpy(c->buffer + left, in, (size_t)ilen);
}
static void md5_variant(const uint8_t* data, uint64_t len, uint8_t out[16]) {
  md5_ctx c;
  c.total[0] = c.total[1] = 0;
  c.state[0] = 0x67452301; c.state[1] = 0xEFCDAB89; c.state[2] = 0x98BADCFE; c.state[3] = 0x10325476;
  if (len > (uint64_t)INT_MAX) {
    uint64_t max = len / 128;
    for (uint64_t i = 0; i < max; i++) {
      int n = 128;
      if (i == max - 1) n = (int)(len % 128);
      md5_update(&c, data + i * 128, n);
    }
  } else {
    md5_update(&c, data, (int)len);
  }
  uint8_t msglen[8];
  uint32_t high = (c.total[0] >> 29) | (c.total[1] << 3), low = c.total[0] << 3;
  for (int i = 0; i < 4; i++) { msglen[i] = (uint8_t)(low >> (8*i)); msglen[4+i] = (uint8_t)(high >> (8*i)); }
  uint32_t last = c.total[0] & 0x3F;
  uint32_t padn = (last < 56) ? (56 - last) : (120 - last);
  static const uint8_t pad[64] = {0x80};
  md5_update(&c, pad, (int)padn);
  md5_update(&c, msglen, 8);
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) out[4*i+j] = (uint8_t)(c.state[i] >> (8*j));
}

static void hash_fn(int kind, const uint8_t* data, uint64_t len, uint8_t out[16]) {
  if (kind == H_MD5) md5_variant(data, len, out); else murmur3_variant(data, len, out);
}

/* ------------------------------------------------------------------------ */
/* Merkle-tree index arithmetic: include/kokkos_merkle_tree.hpp:102-142.     */
/* Exact only for a power-of-two number of leaves; restated as written.      */
/* ------------------------------------------------------------------------ */
static void leaf_range(uint32_t node, uint32_t num_nodes, uint32_t* lo, uint32_t* hi) {
  uint32_t l = 2 * node + 1, r = 2 * node + 2;
  while (l < num_nodes) { l = 2 * l + 1; r = 2 * r + 2; }
  l = (l - 1) / 2; r = (r - 2) / 2;
  if (r > num_nodes) r = num_nodes - 1;
  *lo = l; *hi = r;
}
static uint32_t num_leaf_descendents(uint32_t node, uint32_t num_nodes) { uint32_t l, r; leaf_range(node, num_nodes, &l, &r); return r - l + 1; }
static uint32_t leftmost_leaf(uint32_t node, uint32_t num_nodes) { uint32_t l, r; leaf_range(node, num_nodes, &l, &r); return l; }

/* ------------------------------------------------------------------------ */
/* Digest -> NodeID map with Kokkos::UnorderedMap insert semantics           */
/* (insert-if-absent; include/map_helpers.hpp:105-110).  Slot placement is   */
/* not observable, so any open-addressing table restates it.                 */
/* ------------------------------------------------------------------------ */
typedef struct { uint64_t cap, size; uint8_t* used; digest_t* keys; nodeid_t* vals; } dmap_t;
static int dmap_init(dmap_t* m, uint64_t want) {
  uint64_t cap = 64;
  while (cap < want * 2) cap <<= 1;
  m->cap = cap; m->size = 0;
  m->used = (uint8_t*)calloc(cap, 1);
  m->keys = (digest_t*)malloc(cap * sizeof(digest_t));
  m->vals = (nodeid_t*)malloc(cap * sizeof(nodeid_t));
  return (m->used && m->keys && m->vals) ? 0 : -1;
}
static void dmap_free(dmap_t* m) { free(m->used); free(m->keys); free(m->vals); memset(m, 0, sizeof(*m)); }
static inline uint64_t dslot(const digest_t* k, uint64_t mask) {
  uint64_t a; memcpy(&a, k->d, 8);
  a ^= a >> 29; a *= 0xbf58476d1ce4e5b9ULL; a ^= a >> 32;
  return a & mask;
}
static int64_t dmap_find(const dmap_t* m, const digest_t* k) {
  if (!m->cap) return -1;
  uint64_t mask = m->cap - 1, i = dslot(k, mask);
  while (m->used[i]) { if (!memcmp(m->keys[i].d, k->d, 16)) return (int64_t)i; i = (i + 1) & mask; }
  return -1;
}
static int dmap_grow(dmap_t* m) {
  dmap_t n;
  if (dmap_init(&n, m->cap)) return -1;
  for (uint64_t i = 0; i < m->cap; i++) if (m->used[i]) {
    uint64_t j = dslot(&m->keys[i], n.cap - 1);
    while (n.used[j]) j = (j + 1) & (n.cap - 1);
    n.used[j] = 1; n.keys[j] = m->keys[i]; n.vals[j] = m->vals[i]; n.size++;
  }
  dmap_free(m); *m = n; return 0;
}
/* returns slot index; *inserted = 1 on success(), 0 on existing() */
static int64_t dmap_insert(dmap_t* m, const digest_t* k, nodeid_t v, int* inserted) {
  if ((m->size + 1) * 2 > m->cap && dmap_grow(m)) return -1;
  uint64_t mask = m->cap - 1, i = dslot(k, mask);
  while (m->used[i]) {
    if (!memcmp(m->keys[i].d, k->d, 16)) { *inserted = 0; return (int64_t)i; }
    i = (i + 1) & mask;
  }
  m->used[i] = 1; m->keys[i] = *k; m->vals[i] = v; m->size++;
  *inserted = 1; return (int64_t)i;
}

/* ------------------------------------------------------------------------ */
/* Deduplicator state: the members of TreeDeduplicator / ListDeduplicator /  */
/* BasicDeduplicator / FullDeduplicator (include/{tree,list,basic,full}_approach.hpp). */
/* ------------------------------------------------------------------------ */
typedef struct {
  int approach, hash_kind;
  uint32_t chunk_size, current_id, baseline_id;
  uint64_t data_len;
  uint32_t num_chunks, num_nodes;
  digest_t* tree;      /* tree approach: heap of num_nodes digests */
  digest_t* list;      /* list / basic approach: one digest per chunk */
  uint8_t* changed;    /* basic approach: Kokkos::Bitset changes_bitset */
  uint8_t* labels;
  dmap_t map;
  uint32_t *fo_vec, *sh_vec, fo_len, sh_len;
  uint64_t datasizes[2];
} orc_t;

static uint32_t chunks_of(uint64_t len, uint32_t cs) {
  uint64_t n = len / cs;
  if (n * cs < len) n++;
  return (uint32_t)n;
}

ORC_EXPORT void* orc_create(int approach, int hash_kind, uint32_t chunk_size) {
  if (chunk_size == 0 || approach < A_FULL || approach > A_TREE_LOW_OFFSET) return NULL;
  orc_t* h = (orc_t*)calloc(1, sizeof(orc_t));
  if (!h) return NULL;
  h->approach = approach; h->hash_kind = hash_kind; h->chunk_size = chunk_size;
  return h;
}
static void free_state(orc_t* h) {
  free(h->tree); free(h->list); free(h->changed); free(h->labels); free(h->fo_vec); free(h->sh_vec);
  dmap_free(&h->map);
  h->tree = h->list = NULL; h->changed = h->labels = NULL; h->fo_vec = h->sh_vec = NULL;
}
ORC_EXPORT void orc_destroy(void* p) { if (p) { free_state((orc_t*)p); free(p); } }
ORC_EXPORT uint32_t orc_num_first_ocur(void* p) { return ((orc_t*)p)->fo_len; }
ORC_EXPORT uint32_t orc_num_shift_dupl(void* p) { return ((orc_t*)p)->sh_len; }
ORC_EXPORT uint32_t orc_current_id(void* p) { return ((orc_t*)p)->current_id; }
ORC_EXPORT void orc_datasizes(void* p, uint64_t out[2]) { out[0] = ((orc_t*)p)->datasizes[0]; out[1] = ((orc_t*)p)->datasizes[1]; }
ORC_EXPORT void orc_labels(void* p, uint8_t* out) { orc_t* h = (orc_t*)p; if (h->labels) memcpy(out, h->labels, h->num_nodes); }
ORC_EXPORT void orc_hash(int kind, const uint8_t* data, uint64_t len, uint8_t* out) { hash_fn(kind, data, len, out); }
ORC_EXPORT void orc_free(void* p) { free(p); }

static inline int dsame(const digest_t* a, const digest_t* b) { return !memcmp(a->d, b->d, 16); }
/* value_at(find(k)); a miss (never reached by the labelling) reads as UINT_MAX */
static inline nodeid_t dget(const dmap_t* m, const digest_t* k) {
  int64_t i = dmap_find(m, k);
  if (i < 0) return (nodeid_t){UINT32_MAX, UINT32_MAX};
  return m->vals[i];
}
static inline void hash_pair(orc_t* h, uint32_t node) {
  hash_fn(h->hash_kind, h->tree[2 * node + 1].d, 32, h->tree[node].d);
}

/* level iteration helper: the reference starts one level below the leaves  */
/* and walks up while level_beg <= num_nodes (src/tree_approach.cpp:43-48,   */
/* :124 "intentional unsigned integer underflow").                           */
static void first_level(uint32_t num_nodes, uint32_t* beg, uint32_t* end) {
  uint32_t b = 0, e = 0;
  while (e < num_nodes) { b = 2 * b + 1; e = 2 * e + 2; }
  *beg = b; *end = e;
}

/* TreeDeduplicator::dedup_data_baseline, src/tree_approach.cpp:14-259 */
static int tree_dedup_baseline(orc_t* h, const uint8_t* data, uint64_t data_size) {
  const uint32_t N = h->num_chunks, M = h->num_nodes, cur = h->current_id, cs = h->chunk_size;
  uint8_t* labels = h->labels;
  memset(labels, DONE, M);
  for (uint64_t leaf = N - 1; leaf < M; leaf++) {              /* :57-94 */
    uint32_t nb = cs;
    uint64_t off = (leaf - N + 1) * (uint64_t)cs;
    if (leaf == M - 1) nb = (uint32_t)(data_size - off);
    digest_t dg; hash_fn(h->hash_kind, data + off, nb, dg.d);
    int ins; int64_t idx = dmap_insert(&h->map, &dg, (nodeid_t){(uint32_t)leaf, cur}, &ins);
    if (idx < 0) return ORC_ENOMEM;
    if (dsame(&dg, &h->tree[leaf])) labels[leaf] = FIXED_DUPL;
    else if (ins) labels[leaf] = FIRST_OCUR;
    else {
      nodeid_t* info = &h->map.vals[idx];
      if (info->tree == cur) { if ((uint32_t)leaf < info->node) info->node = (uint32_t)leaf; labels[leaf] = FIRST_OCUR; }
      else labels[leaf] = SHIFT_DUPL;
    }
    h->tree[leaf] = dg;
  }
  for (uint32_t leaf = N - 1; leaf < M; leaf++) {              /* :100-114 */
    if (labels[leaf] == FIRST_OCUR) {
      nodeid_t info = dget(&h->map, &h->tree[leaf]);
      if (info.tree == cur && leaf != info.node) labels[leaf] = SHIFT_DUPL;
    }
  }
  uint32_t beg, end;
  first_level(M, &beg, &end);
  while (beg <= M) {                                             /* :124-145 */
    for (uint64_t node = beg; node <= end; node++) {
      if (node < N - 1) {
        uint32_t l = 2 * node + 1, r = 2 * node + 2;
        if (labels[l] == FIRST_OCUR && labels[r] == FIRST_OCUR) {
          labels[node] = FIRST_OCUR;
          hash_pair(h, node);
          int ins; if (dmap_insert(&h->map, &h->tree[node], (nodeid_t){(uint32_t)node, cur}, &ins) < 0) return ORC_ENOMEM;
        }
        if (node == 0 && labels[0] == FIRST_OCUR) h->fo_vec[h->fo_len++] = 0;
      }
    }
    beg = (beg - 1) / 2; end = (end - 2) / 2;
  }
  first_level(M, &beg, &end);
  while (beg <= M) {                                             /* :155-227 */
    for (uint64_t node = beg; node <= end; node++) {
      if (node < N - 1) {
        uint32_t l = 2 * node + 1, r = 2 * node + 2;
        if (labels[l] != labels[r]) {
          labels[node] = DONE;
          if (labels[l] != FIXED_DUPL && labels[l] != DONE) { if (labels[l] == SHIFT_DUPL) h->sh_vec[h->sh_len++] = l; else h->fo_vec[h->fo_len++] = l; }
          if (labels[r] != FIXED_DUPL && labels[r] != DONE) { if (labels[r] == SHIFT_DUPL) h->sh_vec[h->sh_len++] = r; else h->fo_vec[h->fo_len++] = r; }
        } else if (labels[l] == FIXED_DUPL) {
          labels[node] = FIXED_DUPL;
        } else if (labels[l] == SHIFT_DUPL) {
          /* :202 tests the digest of `node` before it is hashed at :221 */
          if (dmap_find(&h->map, &h->tree[node]) >= 0) labels[node] = SHIFT_DUPL;
          else { labels[node] = DONE; h->sh_vec[h->sh_len++] = l; h->sh_vec[h->sh_len++] = r; }
        }
      }
    }
    for (uint64_t node = beg; node <= end; node++) {             /* :218-224 */
      if (node < N - 1) {
        hash_pair(h, node);
        int ins; if (dmap_insert(&h->map, &h->tree[node], (nodeid_t){(uint32_t)node, cur}, &ins) < 0) return ORC_ENOMEM;
      }
    }
    beg = (beg - 1) / 2; end = (end - 2) / 2;
  }
  return ORC_OK;
}

/* TreeDeduplicator::dedup_data (lowest-offset rule), src/tree_approach.cpp:262-509 */
static int tree_dedup(orc_t* h, const uint8_t* data, uint64_t data_size) {
  const uint32_t N = h->num_chunks, M = h->num_nodes, cur = h->current_id, cs = h->chunk_size;
  uint8_t* labels = h->labels;
  memset(labels, DONE, M);
  for (uint64_t leaf = N - 1; leaf < M; leaf++) {              /* :309-351 */
    uint32_t nb = cs;
    uint64_t off = (leaf - (N - 1)) * (uint64_t)cs;
    if (leaf == M - 1) nb = (uint32_t)(data_size - off);
    digest_t dg; hash_fn(h->hash_kind, data + off, nb, dg.d);
    int ins; int64_t idx = dmap_insert(&h->map, &dg, (nodeid_t){(uint32_t)leaf, cur}, &ins);
    if (idx < 0) return ORC_ENOMEM;
    if (dsame(&dg, &h->tree[leaf])) {
      labels[leaf] = FIXED_DUPL;
    } else if (ins) {
      labels[leaf] = FIRST_OCUR; h->tree[leaf] = dg;
    } else {
      nodeid_t* info = &h->map.vals[idx];
      if (info->tree == cur) { if ((uint32_t)leaf < info->node) info->node = (uint32_t)leaf; labels[leaf] = FIRST_OCUR; }
      else labels[leaf] = SHIFT_DUPL;
      h->tree[leaf] = dg;
    }
  }
  for (uint32_t leaf = N - 1; leaf < M; leaf++) {              /* :356-369 */
    if (labels[leaf] == FIRST_OCUR) {
      nodeid_t info = dget(&h->map, &h->tree[leaf]);
      if (info.tree == cur && leaf != info.node) labels[leaf] = SHIFT_DUPL;
    }
  }
  uint32_t beg, end;
  first_level(M, &beg, &end);
  while (beg <= M) {                                             /* :378-404 */
    for (uint64_t node = beg; node <= end; node++) {
      if (node < N - 1) {
        uint32_t l = 2 * node + 1, r = 2 * node + 2;
        if (labels[l] == FIRST_OCUR && labels[r] == FIRST_OCUR) {
          labels[node] = FIRST_OCUR;
          hash_pair(h, node);
          int ins; if (dmap_insert(&h->map, &h->tree[node], (nodeid_t){(uint32_t)node, cur}, &ins) < 0) return ORC_ENOMEM;
        }
        if (node == 0 && labels[0] == FIRST_OCUR) h->fo_vec[h->fo_len++] = 0;
      }
    }
    beg = (beg - 1) / 2; end = (end - 2) / 2;
  }
  first_level(M, &beg, &end);
  while (beg <= M) {                                             /* :413-477 */
    for (uint64_t node = beg; node <= end; node++) {
      if (node < N - 1) {
        uint32_t l = 2 * node + 1, r = 2 * node + 2;
        if (labels[l] != labels[r]) {
          labels[node] = DONE;
          if (labels[l] != FIXED_DUPL && labels[l] != DONE) { if (labels[l] == SHIFT_DUPL) h->sh_vec[h->sh_len++] = l; else h->fo_vec[h->fo_len++] = l; }
          if (labels[r] != FIXED_DUPL && labels[r] != DONE) { if (labels[r] == SHIFT_DUPL) h->sh_vec[h->sh_len++] = r; else h->fo_vec[h->fo_len++] = r; }
        } else if (labels[l] == FIXED_DUPL) {
          labels[node] = FIXED_DUPL;
        } else if (labels[l] == SHIFT_DUPL) {
          hash_pair(h, node);
          if (dmap_find(&h->map, &h->tree[node]) >= 0) labels[node] = SHIFT_DUPL;
          else { labels[node] = DONE; h->sh_vec[h->sh_len++] = l; h->sh_vec[h->sh_len++] = r; }
        }
      }
    }
    beg = (beg - 1) / 2; end = (end - 2) / 2;
  }
  return ORC_OK;
}

/* dedup_low_offset_ref, include/reference_impl.hpp:16-132: serial labelling, */
/* interior nodes by descending index, roots collected in a std::set          */
/* (ascending), interior digests that were not hashed become zero.           */
static int tree_dedup_ref(orc_t* h, const uint8_t* data, uint64_t data_size) {
  const uint32_t N = h->num_chunks, M = h->num_nodes, cur = h->current_id, cs = h->chunk_size;
  uint8_t* labels = h->labels;
  digest_t* curr = (digest_t*)calloc(M, sizeof(digest_t));
  uint8_t* is_root = (uint8_t*)calloc(M, 1);
  if (!curr || !is_root) { free(curr); free(is_root); return ORC_ENOMEM; }
  memset(labels, DONE, M);
  for (uint32_t leaf = N - 1; leaf < M; leaf++) {              /* :44-71 */
    uint32_t nb = cs;
    uint64_t off = (uint64_t)(leaf - (N - 1)) * cs;
    if (leaf == M - 1) nb = (uint32_t)(data_size - off);
    hash_fn(h->hash_kind, data + off, nb, curr[leaf].d);
    int ins; int64_t idx = dmap_insert(&h->map, &curr[leaf], (nodeid_t){leaf, cur}, &ins);
    if (idx < 0) { free(curr); free(is_root); return ORC_ENOMEM; }
    if (dsame(&h->tree[leaf], &curr[leaf])) labels[leaf] = FIXED_DUPL;
    else if (ins) labels[leaf] = FIRST_OCUR;
    else {
      nodeid_t* info = &h->map.vals[idx];
      if (info->tree == cur) {
        if (info->node > leaf) { labels[leaf] = FIRST_OCUR; labels[info->node] = SHIFT_DUPL; info->node = leaf; }
        else labels[leaf] = SHIFT_DUPL;
      } else labels[leaf] = SHIFT_DUPL;
    }
  }
  for (uint32_t node = N - 2; node < N - 1; node--) {          /* :74-82 */
    uint32_t l = 2 * node + 1, r = 2 * node + 2;
    if (labels[l] == FIRST_OCUR && labels[r] == FIRST_OCUR) {
      labels[node] = FIRST_OCUR;
      hash_fn(h->hash_kind, curr[l].d, 32, curr[node].d);
      int ins; if (dmap_insert(&h->map, &curr[node], (nodeid_t){node, cur}, &ins) < 0) { free(curr); free(is_root); return ORC_ENOMEM; }
    }
  }
  for (uint32_t node = N - 2; node < N - 1; node--) {          /* :83-104 */
    uint32_t l = 2 * node + 1, r = 2 * node + 2;
    if (labels[l] != labels[r]) {
      labels[node] = DONE;
      if (labels[l] != FIXED_DUPL && labels[l] != DONE) is_root[l] = 1;
      if (labels[r] != FIXED_DUPL && labels[r] != DONE) is_root[r] = 1;
    } else if (labels[l] == FIXED_DUPL) {
      labels[node] = FIXED_DUPL;
    } else if (labels[l] == SHIFT_DUPL) {
      hash_fn(h->hash_kind, curr[l].d, 32, curr[node].d);
      if (dmap_find(&h->map, &curr[node]) >= 0) labels[node] = SHIFT_DUPL;
      else { labels[node] = DONE; is_root[l] = 1; is_root[r] = 1; }
    }
  }
  if (labels[0] == FIRST_OCUR) is_root[0] = 1;                 /* :105-106 */
  for (uint32_t root = 0; root < M; root++) {                    /* :109-119 */
    if (!is_root[root] || labels[root] == DONE) continue;
    if (labels[root] == FIRST_OCUR) h->fo_vec[h->fo_len++] = root;
    else if (labels[root] == SHIFT_DUPL) h->sh_vec[h->sh_len++] = root;
  }
  memcpy(h->tree, curr, (size_t)M * sizeof(digest_t));           /* :121 */
  free(curr); free(is_root);
  return ORC_OK;
}

/* Kokkos::BinSort with BinOp1D(max_bins, min, max) and sort_within_bins=false,
 * run by a serial backend: a stable counting sort on
 * bin = (int)(mul * (key - min)), mul = 1 when the integral key range fits the
 * bin count, else max_bins / (max - min).  (Kokkos_Sort / BinOp1D, used at
 * src/tree_approach.cpp:677-687 and src/list_approach.cpp:185-195.)        */
static void bin_sort(uint32_t* vals, const uint32_t* keys, uint32_t n, uint32_t max_bins, uint32_t kmin, uint32_t kmax) {
  if (n == 0) return;
  double range = (double)kmax - (double)kmin;
  double mul = (range <= (double)max_bins) ? 1.0 : (double)max_bins / range;
  uint32_t nb = max_bins + 1;
  uint32_t* cnt = (uint32_t*)calloc((size_t)nb + 1, sizeof(uint32_t));
  uint32_t* bins = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
  uint32_t* out = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
  for (uint32_t i = 0; i < n; i++) { int b = (int)(mul * ((double)keys[i] - (double)kmin)); if (b < 0) b = 0; if ((uint32_t)b >= nb) b = (int)nb - 1; bins[i] = (uint32_t)b; cnt[b + 1]++; }
  for (uint32_t b = 0; b < nb; b++) cnt[b + 1] += cnt[b];
  for (uint32_t i = 0; i < n; i++) out[cnt[bins[i]]++] = vals[i];
  memcpy(vals, out, (size_t)n * sizeof(uint32_t));
  free(cnt); free(bins); free(out);
}

static inline void put32(uint8_t* p, uint32_t v) { memcpy(p, &v, 4); }
static inline uint32_t get32(const uint8_t* p) { uint32_t v; memcpy(&v, p, 4); return v; }

/* TreeDeduplicator::collect_diff, src/tree_approach.cpp:512-710 */
static int tree_collect(orc_t* h, const uint8_t* data, uint64_t data_size, uint8_t** out, uint64_t* out_len, header_t* hd) {
  const uint32_t cs = h->chunk_size, cur = h->current_id;
  const uint32_t N = chunks_of(data_size, cs), M = 2 * N - 1;
  uint32_t F = h->fo_len, S = h->sh_len;
  uint32_t* region_nodes = (uint32_t*)malloc(((size_t)F + 1) * 4);
  uint32_t* region_len = (uint32_t*)malloc(((size_t)F + 1) * 4);
  uint64_t* prior = (uint64_t*)calloc((size_t)cur + 1, 8);
  uint32_t* keys = (uint32_t*)malloc(((size_t)S + 1) * 4);
  if (!region_nodes || !region_len || !prior || !keys) return ORC_ENOMEM;
  uint32_t num_distinct = 0; uint64_t chunk_counter = 0;
  for (uint32_t i = 0; i < F; i++) {                             /* :546-558 */
    uint32_t node = h->fo_vec[i];
    nodeid_t prev = dget(&h->map, &h->tree[node]);
    if (node == prev.node && cur == prev.tree) {
      uint32_t sz = num_leaf_descendents(node, M);
      region_nodes[num_distinct] = node; region_len[num_distinct] = sz; num_distinct++;
      chunk_counter += sz;
    }
  }
  uint32_t P = 0;
  for (uint32_t i = 0; i < S; i++) {                             /* :574-580 */
    nodeid_t prev = dget(&h->map, &h->tree[h->sh_vec[i]]);
    if (prev.tree > cur) return ORC_EINTERNAL;
    if (prior[prev.tree]++ == 0) P++;
  }
  uint64_t data_offset = (uint64_t)F * 4 + (uint64_t)S * 8 + (uint64_t)P * 8;          /* :593 */
  uint64_t run = 0;                                              /* :602-606 */
  for (uint32_t i = 0; i < num_distinct; i++) { uint32_t l = region_len[i]; region_len[i] = (uint32_t)run; run += l; }
  uint64_t buffer_len = 32 + (uint64_t)F * 4 + 8 * (uint64_t)P + (uint64_t)S * 8 + chunk_counter * cs;  /* :622 */
  uint8_t* buf = (uint8_t*)calloc(buffer_len, 1);
  if (!buf) return ORC_ENOMEM;
  for (uint32_t i = 0; i < num_distinct; i++) put32(buf + 32 + 4 * (uint64_t)i, region_nodes[i]);   /* :630-633 */
  for (uint32_t i = 0; i < num_distinct; i++) {                  /* :609-617, :636-650 */
    uint32_t node = region_nodes[i], sz = num_leaf_descendents(node, M);
    uint32_t start = leftmost_leaf(node, M) - (N - 1);
    for (uint32_t j = 0; j < sz; j++) {
      uint64_t slot = (uint64_t)region_len[i] + j;
      uint32_t chunk = start + j;
      uint64_t src = (uint64_t)chunk * cs;
      uint64_t ws = cs;
      if (chunk == N - 1) ws = data_size - src;
      if (src >= data_size) continue;           /* beyond the buffer: the reference reads out of bounds */
      if (src + ws > data_size) ws = data_size - src;
      memcpy(buf + 32 + data_offset + slot * cs, data + src, ws);
    }
  }
  uint64_t pos = 4 * (uint64_t)num_distinct;                     /* :625, :657-665 */
  for (uint32_t i = 0; i <= cur; i++) {
    if (prior[i] > 0) { put32(buf + 32 + pos, i); put32(buf + 32 + pos + 4, (uint32_t)prior[i]); pos += 8; }
  }
  uint64_t prior_start = (uint64_t)num_distinct * 4 + (uint64_t)P * 8;   /* :667 */
  for (uint32_t i = 0; i < S; i++) keys[i] = dget(&h->map, &h->tree[h->sh_vec[i]]).tree;  /* :672-675 */
  bin_sort(h->sh_vec, keys, S, cur, 0, cur);                     /* :677-687 */
  for (uint32_t i = 0; i < S; i++) {                             /* :691-696 */
    uint32_t node = h->sh_vec[i];
    nodeid_t prev = dget(&h->map, &h->tree[node]);
    put32(buf + 32 + prior_start + 8 * (uint64_t)i, node);
    put32(buf + 32 + prior_start + 8 * (uint64_t)i + 4, prev.node);
  }
  hd->ref_id = h->baseline_id; hd->chkpt_id = cur; hd->datalen = data_size; hd->chunk_size = cs;   /* :700-706 */
  hd->num_first_ocur = F; hd->num_shift_dupl = S; hd->num_prior_chkpts = P;
  uint64_t size_meta = (uint64_t)F * 4 + (uint64_t)P * 8 + (uint64_t)S * 8;
  h->datasizes[0] = buffer_len - size_meta; h->datasizes[1] = size_meta;
  free(region_nodes); free(region_len); free(prior); free(keys);
  *out = buf; *out_len = buffer_len;
  return ORC_OK;
}

/* ListDeduplicator::dedup_data, src/list_approach.cpp:23-66 */
static int list_dedup(orc_t* h, const uint8_t* data, uint64_t len) {
  const uint32_t N = h->num_chunks, cs = h->chunk_size, cur = h->current_id;
  for (uint32_t i = 0; i < N; i++) {
    uint32_t nb = cs; uint64_t off = (uint64_t)i * cs;
    if (i == N - 1) nb = (uint32_t)(len - off);
    digest_t dg; hash_fn(h->hash_kind, data + off, nb, dg.d);
    if (!dsame(&h->list[i], &dg)) {
      int ins; if (dmap_insert(&h->map, &dg, (nodeid_t){i, cur}, &ins) < 0) return ORC_ENOMEM;
      if (ins) h->fo_vec[h->fo_len++] = i; else h->sh_vec[h->sh_len++] = i;
      h->list[i] = dg;
    }
  }
  return ORC_OK;
}

/* ListDeduplicator::collect_diff, src/list_approach.cpp:79-247 */
static int list_collect(orc_t* h, const uint8_t* data, uint64_t len, uint8_t** out, uint64_t* out_len, header_t* hd) {
  const uint32_t cs = h->chunk_size, cur = h->current_id, N = chunks_of(h->data_len, cs);
  uint32_t F = h->fo_len, S = h->sh_len, P = 0;
  uint64_t* prior = (uint64_t*)calloc((size_t)cur + 1, 8);
  uint32_t* keys = (uint32_t*)malloc(((size_t)S + 1) * 4);
  if (!prior || !keys) return ORC_ENOMEM;
  for (uint32_t i = 0; i < S; i++) {                             /* :104-109 */
    nodeid_t e = dget(&h->map, &h->list[h->sh_vec[i]]);
    if (e.tree > cur) return ORC_EINTERNAL;
    if (prior[e.tree]++ == 0) P++;
  }
  uint64_t cnt_off = 32 + (uint64_t)F * 4, map_off = cnt_off + (uint64_t)P * 8, data_off = map_off + (uint64_t)S * 8;
  uint64_t size = 32 + (uint64_t)F * (4 + (uint64_t)cs) + (uint64_t)P * 8 + (uint64_t)S * 8;   /* :126-129 */
  uint8_t* buf = (uint8_t*)calloc(size, 1);
  if (!buf) return ORC_ENOMEM;
  for (uint32_t i = 0; i < F; i++) put32(buf + 32 + 4 * (uint64_t)i, h->fo_vec[i]);   /* :141-145 */
  uint64_t pos = cnt_off;                                        /* :149-156 */
  for (uint32_t i = 0; i <= cur; i++) if (prior[i] > 0) { put32(buf + pos, i); put32(buf + pos + 4, (uint32_t)prior[i]); pos += 8; }
  uint32_t max_key = 0;
  for (uint32_t i = 0; i < S; i++) {                             /* :170-182 */
    keys[i] = dget(&h->map, &h->list[h->sh_vec[i]]).tree;
    if (keys[i] > max_key) max_key = keys[i];
  }
  bin_sort(h->sh_vec, keys, S, S, 0, max_key);                   /* :185-195 */
  for (uint32_t i = 0; i < S; i++) {                             /* :199-205 */
    uint32_t node = h->sh_vec[i];
    nodeid_t prev = dget(&h->map, &h->list[node]);
    put32(buf + map_off + 8 * (uint64_t)i, node); put32(buf + map_off + 8 * (uint64_t)i + 4, prev.node);
  }
  for (uint32_t i = 0; i < F; i++) {                             /* :209-223 */
    uint32_t chunk = h->fo_vec[i];
    uint64_t src = (uint64_t)cs * chunk, ws = cs;
    if (chunk == N - 1) ws = h->data_len - src;
    memcpy(buf + data_off + (uint64_t)i * cs, data + src, ws);
  }
  hd->ref_id = h->baseline_id; hd->chkpt_id = cur; hd->datalen = h->data_len; hd->chunk_size = cs;
  hd->num_first_ocur = F; hd->num_shift_dupl = S; hd->num_prior_chkpts = P;
  h->datasizes[0] = (uint64_t)cs * F; h->datasizes[1] = size - (uint64_t)cs * F;
  free(prior); free(keys);
  *out = buf; *out_len = size;
  (void)len;
  return ORC_OK;
}

/* BasicDeduplicator::dedup_data + collect_diff, src/basic_approach.cpp:14-143 */
static int basic_run(orc_t* h, const uint8_t* data, uint64_t len, uint8_t** out, uint64_t* out_len, header_t* hd) {
  const uint32_t N = h->num_chunks, cs = h->chunk_size;
  uint32_t F = 0;
  memset(h->changed, 0, N);
  for (uint32_t i = 0; i < N; i++) {
    uint32_t nb = cs; uint64_t off = (uint64_t)i * cs;
    if (i == N - 1) nb = (uint32_t)(len - off);
    digest_t dg; hash_fn(h->hash_kind, data + off, nb, dg.d);
    if (h->current_id > 0) { if (!dsame(&h->list[i], &dg)) { h->list[i] = dg; h->changed[i] = 1; } }
    else { h->changed[i] = 1; h->list[i] = dg; }
  }
  for (uint32_t i = 0; i < N; i++) F += h->changed[i];
  h->fo_len = F;  /* reported as num_first_ocur (header field) */
  h->sh_len = 0;
  uint64_t size = 32 + (uint64_t)F * (4 + (uint64_t)cs);
  uint8_t* buf = (uint8_t*)calloc(size, 1);
  if (!buf) return ORC_ENOMEM;
  uint64_t data_off = (uint64_t)F * 4, k = 0;
  for (uint32_t i = 0; i < N; i++) {
    if (!h->changed[i]) continue;
    put32(buf + 32 + 4 * k, i);
    uint64_t ws = cs;
    if (i == N - 1) ws = len - (uint64_t)i * cs;
    memcpy(buf + 32 + data_off + k * cs, data + (uint64_t)i * cs, ws);
    k++;
  }
  hd->ref_id = h->baseline_id; hd->chkpt_id = h->current_id; hd->datalen = len; hd->chunk_size = cs;
  hd->num_first_ocur = F; hd->num_shift_dupl = 0; hd->num_prior_chkpts = 0;
  /* :141-142 multiply num_first_ocur * chunk_size in 32 bits */
  uint32_t dsz = F * cs;
  h->datasizes[0] = dsz; h->datasizes[1] = size - dsz;
  *out = buf; *out_len = size;
  return ORC_OK;
}

/* checkpoint(header_t&, ...) of each approach: src/tree_approach.cpp:1578-1689,
 * src/list_approach.cpp:843-931, src/basic_approach.cpp:468-549,
 * src/full_approach.cpp:14-77.  `increment` selects the convenience
 * overloads, which add 1 to current_id afterwards (:1723, :1747, :1775).   */
ORC_EXPORT int orc_checkpoint(void* p, const uint8_t* data, uint64_t len, int make_baseline, int increment,
                              uint8_t** out, uint64_t* out_len) {
  orc_t* h = (orc_t*)p;
  if (!h || !out || !out_len || len == 0) return ORC_EINVAL;
  const uint32_t cs = h->chunk_size;
  uint32_t N = chunks_of(len, cs), M = 2 * N - 1;
  header_t hd; memset(&hd, 0, sizeof(hd));
  int rc = ORC_OK;
  if (h->approach == A_FULL) {
    uint8_t* buf = (uint8_t*)malloc(len);
    if (!buf) return ORC_ENOMEM;
    memcpy(buf, data, len);
    h->data_len = len; h->datasizes[0] = len; h->datasizes[1] = 0;
    *out = buf; *out_len = len;
    if (increment) h->current_id++;
    return ORC_OK;
  }
  /* state is (re)allocated only for a baseline or on first use, as the
   * reference does under `if(make_baseline)` (src/tree_approach.cpp:1601-1606) */
  int fresh = make_baseline || !h->fo_vec;
  if (!fresh && len != h->data_len) return ORC_EINVAL;   /* length changes need a new baseline */
  if (fresh) {
    free_state(h);
    h->num_chunks = N; h->num_nodes = M; h->data_len = len;
    if (h->approach == A_LIST || h->approach == A_BASIC) {
      h->list = (digest_t*)calloc(N, sizeof(digest_t));
      h->changed = (uint8_t*)calloc(N, 1);
      if (!h->list || !h->changed) return ORC_ENOMEM;
      if (h->approach == A_LIST && dmap_init(&h->map, N)) return ORC_ENOMEM;
    } else {
      h->tree = (digest_t*)calloc(M, sizeof(digest_t));
      h->labels = (uint8_t*)malloc(M);
      if (!h->tree || !h->labels || dmap_init(&h->map, M)) return ORC_ENOMEM;
    }
    h->fo_vec = (uint32_t*)malloc((size_t)N * 8 + 8);
    h->sh_vec = (uint32_t*)malloc((size_t)N * 8 + 8);
    if (!h->fo_vec || !h->sh_vec) return ORC_ENOMEM;
  }
  h->fo_len = h->sh_len = 0;
  if (h->current_id == 0 || make_baseline) h->baseline_id = h->current_id;
  if (h->approach == A_BASIC) {
    rc = basic_run(h, data, len, out, out_len, &hd);
  } else if (h->approach == A_LIST) {
    rc = list_dedup(h, data, len);
    if (rc == ORC_OK) rc = list_collect(h, data, len, out, out_len, &hd);
  } else {
    if (h->approach == A_TREE_REF) rc = tree_dedup_ref(h, data, len);
    else if (h->current_id == 0 || make_baseline) rc = tree_dedup_baseline(h, data, len);
    else rc = tree_dedup(h, data, len);
    if (rc == ORC_OK) rc = tree_collect(h, data, len, out, out_len, &hd);
  }
  if (rc != ORC_OK) return rc;
  memcpy(*out, &hd, sizeof(hd));
  if (increment) h->current_id++;
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Restart.                                                                  */
/* ------------------------------------------------------------------------ */
typedef struct { header_t h; const uint8_t* buf; uint64_t size, fo_off, cnt_off, map_off, data_off; } diffview_t;
static int parse(const uint8_t* buf, uint64_t size, diffview_t* v, int basic) {
  if (size < 32) return ORC_ECORRUPT;
  memcpy(&v->h, buf, 32);
  v->buf = buf; v->size = size;
  if (v->h.chunk_size == 0) return ORC_ECORRUPT;
  v->fo_off = 32;
  v->cnt_off = 32 + 4 * (uint64_t)v->h.num_first_ocur;
  v->map_off = v->cnt_off + (basic ? 0 : 8 * (uint64_t)v->h.num_prior_chkpts);
  v->data_off = v->map_off + (basic ? 0 : 8 * (uint64_t)v->h.num_shift_dupl);
  if (v->data_off > size) return ORC_ECORRUPT;
  return ORC_OK;
}
/* bounded copy out of a diff's data section into the restart buffer */
static void copy_out(uint8_t* out, uint64_t out_len, uint64_t dst, const diffview_t* v, uint64_t src, uint64_t n) {
  if (dst >= out_len) return;
  if (dst + n > out_len) n = out_len - dst;
  uint64_t s = v->data_off + src;
  if (s >= v->size) return;
  if (s + n > v->size) n = v->size - s;
  memcpy(out + dst, v->buf + s, n);
}
/* repeat-count table -> inclusive prefix over checkpoint ids (:872-883) */
static int load_repeat_sizes(const diffview_t* v, uint32_t cur, uint32_t* rrs) {
  memset(rrs, 0, ((size_t)cur + 1) * 4);
  for (uint32_t i = 0; i < v->h.num_prior_chkpts; i++) {
    uint32_t ck = get32(v->buf + v->cnt_off + 8 * (uint64_t)i);
    if (ck > cur) return ORC_ECORRUPT;
    rrs[ck] = get32(v->buf + v->cnt_off + 8 * (uint64_t)i + 4);
  }
  uint32_t s = 0;
  for (uint32_t i = 0; i <= cur; i++) { s += rrs[i]; rrs[i] = s; }
  return ORC_OK;
}
static uint32_t source_tree(const uint32_t* rrs, uint32_t cur, uint32_t i) {
  uint32_t tree = 0;
  for (uint32_t j = cur; j <= cur; j--) if (i < rrs[j]) tree = j;   /* :894-898 */
  return tree;
}

/* node-id keyed first-wins maps over [0, num_nodes] (Kokkos::UnorderedMap<NodeID,size_t> / <uint32_t,NodeID>) */
typedef struct { uint64_t n; uint8_t* has; uint64_t* val; } offmap_t;
typedef struct { uint64_t n; uint8_t* has; nodeid_t* val; } idmap_t;

/* TreeDeduplicator::restart_chkpt, src/tree_approach.cpp:713-1128 */
static int tree_restart(const uint8_t* const* diffs, const uint64_t* lens, uint32_t ndiffs, uint32_t idx0, uint8_t* out, uint64_t out_len) {
  diffview_t v;
  int rc = parse(diffs[idx0], lens[idx0], &v, 0);
  if (rc) return rc;
  if (v.h.datalen != out_len) return ORC_EINVAL;
  const uint32_t N = chunks_of(v.h.datalen, v.h.chunk_size), M = 2 * N - 1;
  uint64_t datalen = v.h.datalen; uint32_t cs = v.h.chunk_size, cur = v.h.chkpt_id, ref_id = v.h.ref_id;
  nodeid_t* node_list = (nodeid_t*)malloc((size_t)N * sizeof(nodeid_t));
  offmap_t dm = { (uint64_t)M + 2, (uint8_t*)calloc((size_t)M + 2, 1), (uint64_t*)malloc(((size_t)M + 2) * 8) };
  idmap_t rm = { (uint64_t)M + 2, (uint8_t*)calloc((size_t)M + 2, 1), (nodeid_t*)malloc(((size_t)M + 2) * sizeof(nodeid_t)) };
  uint32_t* rrs = NULL;
  uint32_t* chunk_len = NULL;
  if (!node_list || !dm.has || !dm.val || !rm.has || !rm.val) { rc = ORC_ENOMEM; goto done; }
  for (uint32_t i = 0; i < N; i++) node_list[i] = (nodeid_t){UINT32_MAX, UINT32_MAX};
  {
    uint32_t F = v.h.num_first_ocur, S = v.h.num_shift_dupl;
    chunk_len = (uint32_t*)malloc(((size_t)F + 1) * 4);
    rrs = (uint32_t*)malloc(((size_t)cur + 2) * 4);
    if (!chunk_len || !rrs) { rc = ORC_ENOMEM; goto done; }
    uint32_t run = 0;                                            /* :803-816 */
    for (uint32_t i = 0; i < F; i++) { uint32_t node = get32(v.buf + 32 + 4 * (uint64_t)i); chunk_len[i] = run; run += num_leaf_descendents(node, M); }
    for (uint32_t i = 0; i < F; i++) {                           /* :825-865 */
      uint32_t node = get32(v.buf + 32 + 4 * (uint64_t)i);
      if (node > M) { rc = ORC_ECORRUPT; goto done; }
      if (!dm.has[node]) { dm.has[node] = 1; dm.val[node] = (uint64_t)chunk_len[i] * cs; }
      uint32_t start = leftmost_leaf(node, M), len = num_leaf_descendents(node, M), end = start + len - 1;
      uint32_t left = 2 * node + 1, right = 2 * node + 2;
      while (left < M) {
        if (right >= M) right = M;
        for (uint32_t u = left; u <= right; u++) {
          uint32_t leaf = leftmost_leaf(u, M);
          if (!dm.has[u]) { dm.has[u] = 1; dm.val[u] = (uint64_t)(chunk_len[i] + leaf - start) * cs; }
        }
        left = 2 * left + 1; right = 2 * right + 2;
      }
      for (uint32_t j = 0; j < len; j++) { uint32_t c = start - N + 1 + j; if (c < N) node_list[c] = (nodeid_t){c, cur}; }
      uint64_t src = (uint64_t)chunk_len[i] * cs, dst = (uint64_t)(start - N + 1) * cs, n = (uint64_t)len * cs;
      if (end == M - 1) n = datalen - dst;
      copy_out(out, out_len, dst, &v, src, n);
    }
    if ((rc = load_repeat_sizes(&v, cur, rrs))) goto done;       /* :868-883 */
    for (uint32_t i = 0; i < S; i++) {                           /* :887-925 */
      uint32_t node = get32(v.buf + v.map_off + 8 * (uint64_t)i), prev = get32(v.buf + v.map_off + 8 * (uint64_t)i + 4);
      if (node > M || prev > M) { rc = ORC_ECORRUPT; goto done; }
      uint32_t tree = source_tree(rrs, cur, i);
      uint64_t offset = 0;
      if (tree == cur && dm.has[prev]) offset = dm.val[prev];
      uint32_t node_start = leftmost_leaf(node, M), prev_start = leftmost_leaf(prev, M), len = num_leaf_descendents(prev, M);
      for (uint32_t j = 0; j < len; j++) { uint32_t c = node_start + j - N + 1; if (c < N) node_list[c] = (nodeid_t){prev_start + j, tree}; }
      if (tree == cur) {
        uint64_t dst = (uint64_t)cs * (node_start - N + 1), n = (uint64_t)cs * len;
        if (node_start + len - 1 == M - 1) n = datalen - dst;
        copy_out(out, out_len, dst, &v, offset, n);
      }
    }
    for (uint32_t i = 0; i < N; i++) if (node_list[i].node == UINT32_MAX) node_list[i] = (nodeid_t){i + N - 1, cur - 1};   /* :932-937 */
  }
  for (int idx = (int)idx0 - 1; idx >= (int)ref_id; idx--) {     /* :943-1121 */
    if ((uint32_t)idx >= ndiffs) { rc = ORC_EINVAL; goto done; }
    diffview_t c;
    if ((rc = parse(diffs[idx], lens[idx], &c, 0))) goto done;
    ref_id = c.h.ref_id; cur = c.h.chkpt_id; datalen = c.h.datalen; cs = c.h.chunk_size;
    uint32_t F = c.h.num_first_ocur, S = c.h.num_shift_dupl;
    memset(dm.has, 0, (size_t)dm.n); memset(rm.has, 0, (size_t)rm.n);
    free(chunk_len); free(rrs);
    chunk_len = (uint32_t*)malloc(((size_t)F + 1) * 4);
    rrs = (uint32_t*)malloc(((size_t)cur + 2) * 4);
    if (!chunk_len || !rrs) { rc = ORC_ENOMEM; goto done; }
    uint32_t run = 0;
    for (uint32_t i = 0; i < F; i++) { uint32_t node = get32(c.buf + 32 + 4 * (uint64_t)i); chunk_len[i] = run; run += num_leaf_descendents(node, M); }
    for (uint32_t i = 0; i < F; i++) {                           /* :1017-1041 */
      uint32_t node = get32(c.buf + 32 + 4 * (uint64_t)i);
      if (node > M) { rc = ORC_ECORRUPT; goto done; }
      uint64_t offset = (uint64_t)chunk_len[i] * cs;
      if (!dm.has[node]) { dm.has[node] = 1; dm.val[node] = offset; }
      uint32_t start = leftmost_leaf(node, M), left = 2 * node + 1, right = 2 * node + 2;
      while (left < M) {
        if (right >= M) right = M;
        for (uint32_t u = left; u <= right; u++) {
          uint32_t leaf = leftmost_leaf(u, M);
          if (!dm.has[u]) { dm.has[u] = 1; dm.val[u] = offset + (uint64_t)(leaf - start) * cs; }
        }
        left = 2 * left + 1; right = 2 * right + 2;
      }
    }
    if ((rc = load_repeat_sizes(&c, cur, rrs))) goto done;
    for (uint32_t i = 0; i < S; i++) {                           /* :1058-1079 */
      uint32_t node = get32(c.buf + c.map_off + 8 * (uint64_t)i), prev = get32(c.buf + c.map_off + 8 * (uint64_t)i + 4);
      if (node > M || prev > M) { rc = ORC_ECORRUPT; goto done; }
      uint32_t tree = source_tree(rrs, cur, i);
      if (!rm.has[node]) { rm.has[node] = 1; rm.val[node] = (nodeid_t){prev, tree}; }
      uint32_t cstart = leftmost_leaf(node, M), pstart = leftmost_leaf(prev, M), len = num_leaf_descendents(node, M);
      for (uint32_t u = 0; u < len; u++) {
        uint32_t k = cstart + u;
        if (k <= M && !rm.has[k]) { rm.has[k] = 1; rm.val[k] = (nodeid_t){pstart + u, tree}; }
      }
    }
    for (uint32_t i = 0; i < N; i++) {                           /* :1083-1118 */
      if (node_list[i].tree != cur) continue;
      nodeid_t id = node_list[i];
      uint64_t dst = (uint64_t)i * cs, ws = cs;
      if (dst + ws > datalen) ws = datalen - dst;
      if (id.node <= M && dm.has[id.node]) {
        copy_out(out, out_len, dst, &c, dm.val[id.node], ws);
      } else if (id.node <= M && rm.has[id.node]) {
        nodeid_t prev = rm.val[id.node];
        if (prev.tree == cur) {
          if (prev.node <= M && dm.has[prev.node]) copy_out(out, out_len, dst, &c, dm.val[prev.node], ws);
        } else node_list[i] = prev;
      } else {
        node_list[i] = (nodeid_t){id.node, cur - 1};
      }
    }
  }
done:
  free(node_list); free(dm.has); free(dm.val); free(rm.has); free(rm.val); free(rrs); free(chunk_len);
  return rc;
}

/* ListDeduplicator::restart_chkpt, src/list_approach.cpp:259-574 */
static int list_restart(const uint8_t* const* diffs, const uint64_t* lens, uint32_t ndiffs, uint32_t idx0, uint8_t* out, uint64_t out_len) {
  diffview_t v;
  int rc = parse(diffs[idx0], lens[idx0], &v, 0);
  if (rc) return rc;
  if (v.h.datalen != out_len) return ORC_EINVAL;
  const uint32_t N = chunks_of(v.h.datalen, v.h.chunk_size);
  uint64_t datalen = v.h.datalen; uint32_t cs = v.h.chunk_size, cur = v.h.chkpt_id, ref_id = v.h.ref_id;
  nodeid_t* node_list = (nodeid_t*)malloc((size_t)N * sizeof(nodeid_t));
  uint8_t* fo_has = (uint8_t*)calloc(N, 1); uint64_t* fo_val = (uint64_t*)malloc((size_t)N * 8);
  uint8_t* rm_has = (uint8_t*)calloc(N, 1); nodeid_t* rm_val = (nodeid_t*)malloc((size_t)N * sizeof(nodeid_t));
  uint32_t* rrs = NULL;
  if (!node_list || !fo_has || !fo_val || !rm_has || !rm_val) { rc = ORC_ENOMEM; goto done; }
  for (uint32_t i = 0; i < N; i++) node_list[i] = (nodeid_t){UINT32_MAX, UINT32_MAX};
  for (uint32_t i = 0; i < v.h.num_first_ocur; i++) {            /* :326-348 */
    uint32_t node = get32(v.buf + 32 + 4 * (uint64_t)i);
    if (node >= N) { rc = ORC_ECORRUPT; goto done; }
    if (!fo_has[node]) { fo_has[node] = 1; fo_val[node] = (uint64_t)i * cs; }
    node_list[node] = (nodeid_t){node, cur};
    uint64_t dst = (uint64_t)node * cs, ws = cs;
    if (node == N - 1) ws = datalen - dst;
    copy_out(out, out_len, dst, &v, (uint64_t)i * cs, ws);
  }
  rrs = (uint32_t*)malloc(((size_t)cur + 2) * 4);
  if (!rrs) { rc = ORC_ENOMEM; goto done; }
  if ((rc = load_repeat_sizes(&v, cur, rrs))) goto done;         /* :350-369 */
  for (uint32_t i = 0; i < v.h.num_shift_dupl; i++) {            /* :376-411 */
    uint32_t node = get32(v.buf + v.map_off + 8 * (uint64_t)i), prev = get32(v.buf + v.map_off + 8 * (uint64_t)i + 4);
    if (node >= N) { rc = ORC_ECORRUPT; goto done; }
    uint32_t tree = source_tree(rrs, cur, i);
    uint64_t src = 0;
    if (tree == cur && prev < N && fo_has[prev]) src = fo_val[prev];
    node_list[node] = (nodeid_t){prev, tree};
    if (tree == cur) {
      uint64_t dst = (uint64_t)node * cs, ws = cs;
      if (node == N - 1) ws = datalen - dst;
      copy_out(out, out_len, dst, &v, src, ws);
    }
  }
  for (uint32_t i = 0; i < N; i++) if (node_list[i].node == UINT32_MAX) node_list[i] = (nodeid_t){i, cur - 1};   /* :417-422 */
  for (int idx = (int)idx0 - 1; idx >= (int)ref_id && idx < (int)idx0; idx--) {   /* :428-568 */
    if ((uint32_t)idx >= ndiffs) { rc = ORC_EINVAL; goto done; }
    diffview_t c;
    if ((rc = parse(diffs[idx], lens[idx], &c, 0))) goto done;
    uint32_t current_id = c.h.chkpt_id;
    ref_id = c.h.ref_id; cur = c.h.chkpt_id; datalen = c.h.datalen; cs = c.h.chunk_size;
    memset(fo_has, 0, N); memset(rm_has, 0, N);
    for (uint32_t i = 0; i < c.h.num_first_ocur; i++) {
      uint32_t node = get32(c.buf + 32 + 4 * (uint64_t)i);
      if (node >= N) { rc = ORC_ECORRUPT; goto done; }
      if (!fo_has[node]) { fo_has[node] = 1; fo_val[node] = (uint64_t)i * cs; }
    }
    free(rrs); rrs = (uint32_t*)malloc(((size_t)cur + 2) * 4);
    if (!rrs) { rc = ORC_ENOMEM; goto done; }
    if ((rc = load_repeat_sizes(&c, cur, rrs))) goto done;
    for (uint32_t i = 0; i < c.h.num_shift_dupl; i++) {
      uint32_t node = get32(c.buf + c.map_off + 8 * (uint64_t)i), prev = get32(c.buf + c.map_off + 8 * (uint64_t)i + 4);
      if (node >= N) { rc = ORC_ECORRUPT; goto done; }
      if (!rm_has[node]) { rm_has[node] = 1; rm_val[node] = (nodeid_t){prev, source_tree(rrs, cur, i)}; }
    }
    for (uint32_t i = 0; i < N; i++) {
      if (node_list[i].tree != current_id) continue;
      nodeid_t id = node_list[i];
      uint64_t dst = (uint64_t)i * cs, ws = cs;
      if (dst + ws > datalen) ws = datalen - dst;
      /* the lookup key is the pair (node, tree); tree == current_id here */
      if (id.node < N && fo_has[id.node]) {
        copy_out(out, out_len, dst, &c, fo_val[id.node], ws);
      } else if (id.node < N && rm_has[id.node]) {
        nodeid_t prev = rm_val[id.node];
        if (prev.tree == current_id) {
          if (prev.node < N && fo_has[prev.node]) copy_out(out, out_len, dst, &c, fo_val[prev.node], ws);
        } else node_list[i] = prev;
      } else {
        node_list[i] = (nodeid_t){id.node, current_id - 1};
      }
    }
  }
done:
  free(node_list); free(fo_has); free(fo_val); free(rm_has); free(rm_val); free(rrs);
  return rc;
}

/* BasicDeduplicator::restart_chkpt, src/basic_approach.cpp:155-321 */
static int basic_restart(const uint8_t* const* diffs, const uint64_t* lens, uint32_t ndiffs, uint32_t idx0, uint8_t* out, uint64_t out_len) {
  diffview_t v;
  int rc = parse(diffs[idx0], lens[idx0], &v, 1);
  if (rc) return rc;
  if (v.h.datalen != out_len) return ORC_EINVAL;
  const uint32_t N = chunks_of(v.h.datalen, v.h.chunk_size);
  uint64_t datalen = v.h.datalen; uint32_t cs = v.h.chunk_size, cur = v.h.chkpt_id, ref_id = v.h.ref_id;
  nodeid_t* node_list = (nodeid_t*)malloc((size_t)N * sizeof(nodeid_t));
  uint8_t* has = (uint8_t*)calloc(N, 1); uint64_t* val = (uint64_t*)malloc((size_t)N * 8);
  if (!node_list || !has || !val) { rc = ORC_ENOMEM; goto done; }
  for (uint32_t i = 0; i < N; i++) node_list[i] = (nodeid_t){UINT32_MAX, UINT32_MAX};
  for (uint32_t i = 0; i < v.h.num_first_ocur; i++) {            /* :215-235 */
    uint32_t node = get32(v.buf + 32 + 4 * (uint64_t)i);
    if (node >= N) { rc = ORC_ECORRUPT; goto done; }
    node_list[node] = (nodeid_t){node, cur};
    uint64_t dst = (uint64_t)node * cs, ws = cs;
    if (node == N - 1) ws = datalen - dst;
    copy_out(out, out_len, dst, &v, (uint64_t)i * cs, ws);
  }
  for (uint32_t i = 0; i < N; i++) if (node_list[i].node == UINT32_MAX) node_list[i] = (nodeid_t){i, cur - 1};
  for (int idx = (int)idx0 - 1; idx >= (int)ref_id; idx--) {     /* :247-313 */
    if ((uint32_t)idx >= ndiffs) { rc = ORC_EINVAL; goto done; }
    diffview_t c;
    if ((rc = parse(diffs[idx], lens[idx], &c, 1))) goto done;
    ref_id = c.h.ref_id; cur = c.h.chkpt_id; datalen = c.h.datalen; cs = c.h.chunk_size;
    memset(has, 0, N);
    for (uint32_t i = 0; i < c.h.num_first_ocur; i++) {
      uint32_t node = get32(c.buf + 32 + 4 * (uint64_t)i);
      if (node >= N) { rc = ORC_ECORRUPT; goto done; }
      if (!has[node]) { has[node] = 1; val[node] = (uint64_t)i * cs; }
    }
    for (uint32_t i = 0; i < N; i++) {
      if (node_list[i].tree != cur) continue;
      if (node_list[i].node == i && has[i]) {
        uint64_t ws = cs;
        if (i == N - 1) ws = datalen - (uint64_t)i * cs;
        copy_out(out, out_len, (uint64_t)i * cs, &c, val[i], ws);
      } else {
        node_list[i] = (nodeid_t){i, cur - 1};
      }
    }
  }
done:
  free(node_list); free(has); free(val);
  return rc;
}

/* restart(View, std::vector<HostMirror>&, logname, chkpt_id) of each approach;
 * the full approach copies the raw checkpoint (src/full_approach.cpp:122-141). */
ORC_EXPORT int orc_restart(int approach, const uint8_t* const* diffs, const uint64_t* lens, uint32_t n, uint32_t id,
                           uint8_t* out, uint64_t out_len) {
  if (!diffs || !lens || id >= n || !out) return ORC_EINVAL;
  switch (approach) {
    case A_FULL:
      if (lens[id] != out_len) return ORC_EINVAL;
      memcpy(out, diffs[id], out_len);
      return ORC_OK;
    case A_BASIC: return basic_restart(diffs, lens, n, id, out, out_len);
    case A_LIST: return list_restart(diffs, lens, n, id, out, out_len);
    case A_TREE: case A_TREE_REF: case A_TREE_LOW_OFFSET: return tree_restart(diffs, lens, n, id, out, out_len);
    default: return ORC_EINVAL;
  }
}
