// Kokkos_UnorderedMap.hpp -- serial stand-in (test infrastructure; see
// Kokkos_Core.hpp).  An insert-if-absent open-addressing table with linear
// probing; a shallow handle like the Kokkos map.
#pragma once
#include "Kokkos_Bitset.hpp"
#include "Kokkos_Core.hpp"

namespace Kokkos {

template <class K>
struct pod_hash {
  uint32_t operator()(const K& k) const {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&k);
    uint32_t h = 2166136261u;
    for (size_t i = 0; i < sizeof(K); i++) h = (h ^ p[i]) * 16777619u;
    return h;
  }
};
template <class K>
struct pod_equal_to {
  bool operator()(const K& a, const K& b) const { return std::memcmp(&a, &b, sizeof(K)) == 0; }
};

struct UnorderedMapInsertResult {
  enum Status { SUCCESS, EXISTING, FAILED };
  Status st = FAILED;
  uint32_t idx = ~0u;
  bool success() const { return st == SUCCESS; }
  bool existing() const { return st == EXISTING; }
  bool failed() const { return st == FAILED; }
  uint32_t index() const { return idx; }
};

template <class K, class V, class Space = DefaultExecutionSpace, class Hasher = pod_hash<K>,
          class Equal = pod_equal_to<K>>
class UnorderedMap {
  struct Table {
    std::vector<K> keys;
    std::vector<V> vals;
    std::vector<char> used;
    uint32_t size = 0;
  };
  std::shared_ptr<Table> t_;

 public:
  using key_type = K;
  using value_type = V;
  static constexpr uint32_t invalid_index = ~0u;

  UnorderedMap() : UnorderedMap(0) {}
  explicit UnorderedMap(uint32_t capacity) : t_(std::make_shared<Table>()) { resize_table(capacity); }

  void resize_table(uint32_t capacity) {
    uint32_t c = capacity < 16 ? 16 : capacity;
    t_->keys.assign(c, K());
    t_->vals.assign(c, V());
    t_->used.assign(c, 0);
    t_->size = 0;
  }
  uint32_t capacity() const { return (uint32_t)t_->used.size(); }
  uint32_t size() const { return t_->size; }
  void clear() {
    std::fill(t_->used.begin(), t_->used.end(), 0);
    t_->size = 0;
  }
  bool rehash(uint32_t n) {
    if (n < t_->size) n = t_->size;
    Table old = *t_;
    resize_table(n);
    for (uint32_t i = 0; i < old.used.size(); i++)
      if (old.used[i]) insert(old.keys[i], old.vals[i]);
    return true;
  }
  UnorderedMapInsertResult insert(const K& k, const V& v = V()) const {
    UnorderedMapInsertResult r;
    const uint32_t c = capacity();
    uint32_t i = Hasher()(k) % c;
    for (uint32_t probe = 0; probe < c; probe++, i = (i + 1) % c) {
      if (!t_->used[i]) {
        t_->used[i] = 1;
        t_->keys[i] = k;
        t_->vals[i] = v;
        t_->size++;
        r.st = UnorderedMapInsertResult::SUCCESS;
        r.idx = i;
        return r;
      }
      if (Equal()(t_->keys[i], k)) {
        r.st = UnorderedMapInsertResult::EXISTING;
        r.idx = i;
        return r;
      }
    }
    return r;
  }
  uint32_t find(const K& k) const {
    const uint32_t c = capacity();
    uint32_t i = Hasher()(k) % c;
    for (uint32_t probe = 0; probe < c; probe++, i = (i + 1) % c) {
      if (!t_->used[i]) return invalid_index;
      if (Equal()(t_->keys[i], k)) return i;
    }
    return invalid_index;
  }
  bool exists(const K& k) const { return find(k) != invalid_index; }
  bool valid_at(uint32_t i) const { return i < capacity() && t_->used[i]; }
  K& key_at(uint32_t i) const { return t_->keys[i]; }
  // a miss reads a default value (the reference never reads one on its path)
  V& value_at(uint32_t i) const {
    static thread_local V miss;
    if (i >= capacity()) {
      miss = V();
      return miss;
    }
    return t_->vals[i];
  }
  bool failed_insert() const { return false; }
  // deep_copy: this map's table becomes a copy of the other's (same
  // capacity and slots), seen through every handle of this map
  template <class M>
  void assign_from(const M& o) const {
    const uint32_t c = o.capacity();
    t_->keys.assign(c, K());
    t_->vals.assign(c, V());
    t_->used.assign(c, 0);
    t_->size = o.size();
    for (uint32_t i = 0; i < c; i++)
      if (o.valid_at(i)) {
        t_->used[i] = 1;
        t_->keys[i] = o.key_at(i);
        t_->vals[i] = o.value_at(i);
      }
  }
};

template <class K, class V, class S1, class H1, class E1, class S2, class H2, class E2>
void deep_copy(const UnorderedMap<K, V, S1, H1, E1>& dst, const UnorderedMap<K, V, S2, H2, E2>& src) {
  dst.assign_from(src);
}

}  // namespace Kokkos
