// Kokkos_Bitset.hpp -- serial stand-in (test infrastructure; see Kokkos_Core.hpp).
#pragma once
#include "Kokkos_Core.hpp"

namespace Kokkos {
template <class Space = DefaultExecutionSpace>
class Bitset {
  std::shared_ptr<std::vector<char>> b_;

 public:
  Bitset() : b_(std::make_shared<std::vector<char>>()) {}
  explicit Bitset(uint32_t n) : b_(std::make_shared<std::vector<char>>(n, 0)) {}
  uint32_t size() const { return (uint32_t)b_->size(); }
  bool set(uint32_t i) const {
    const bool was = (*b_)[i];
    (*b_)[i] = 1;
    return !was;
  }
  bool reset(uint32_t i) const {
    const bool was = (*b_)[i];
    (*b_)[i] = 0;
    return was;
  }
  void reset() const { std::fill(b_->begin(), b_->end(), 0); }
  void clear() const { reset(); }
  void set() const { std::fill(b_->begin(), b_->end(), 1); }
  bool test(uint32_t i) const { return (*b_)[i] != 0; }
  uint32_t count() const { return (uint32_t)std::count(b_->begin(), b_->end(), 1); }
};
}  // namespace Kokkos
