// Kokkos_Sort.hpp -- serial stand-in for BinSort / BinOp1D (test
// infrastructure; see Kokkos_Core.hpp).  BinOp1D(max_bins, min, max) puts key
// k in bin int(mul * (k - min)), mul = 1 when the keys are integers whose
// range fits max_bins, else max_bins / (max - min), with max_bins + 1 bins
// (Kokkos 3.7 and later).  create_permute_vector() visits the keys in
// ascending index order, as a serial backend does, so each bin keeps the
// keys' original order.
#pragma once
#include "Kokkos_Core.hpp"

namespace Kokkos {

template <class KeyView>
struct BinOp1D {
  using key_type = typename KeyView::non_const_value_type;
  int max_bins_ = 1;
  double mul_ = 1.0;
  double min_ = 0;
  BinOp1D() = default;
  BinOp1D(int max_bins, key_type min, key_type max)
      : max_bins_(max_bins + 1),
        mul_(std::is_integral<key_type>::value && ((double)max - (double)min) <= (double)max_bins
                 ? 1.0
                 : (double)max_bins / ((double)max - (double)min)),
        min_((double)min) {}
  template <class V>
  int bin(const V& keys, size_t i) const {
    return int(mul_ * ((double)keys(i) - min_));
  }
  int max_bins() const { return max_bins_; }
};

template <class KeyView, class BinOp, class Space = DefaultExecutionSpace, class SizeType = size_t>
class BinSort {
  KeyView keys_;
  size_t begin_, end_;
  BinOp op_;
  std::vector<size_t> perm_;

 public:
  BinSort(const KeyView& keys, size_t begin, size_t end, BinOp op, bool /*sort_within_bins*/ = false)
      : keys_(keys), begin_(begin), end_(end), op_(op) {}
  BinSort(const KeyView& keys, BinOp op, bool sort_within_bins = false)
      : BinSort(keys, 0, keys.extent(0), op, sort_within_bins) {}
  void create_permute_vector() {
    const int nb = op_.max_bins();
    std::vector<size_t> count(nb + 1, 0);
    std::vector<int> bins(end_ - begin_);
    for (size_t i = begin_; i < end_; i++) {
      int b = op_.bin(keys_, i);
      bins[i - begin_] = b;
      count[b + 1]++;
    }
    for (int b = 0; b < nb; b++) count[b + 1] += count[b];
    perm_.assign(end_ - begin_, 0);
    for (size_t i = begin_; i < end_; i++) perm_[count[bins[i - begin_]]++] = i;
  }
  template <class V>
  void sort(const V& values) const {
    std::vector<typename V::non_const_value_type> tmp(perm_.size());
    for (size_t k = 0; k < perm_.size(); k++) tmp[k] = values(perm_[k]);
    for (size_t k = 0; k < perm_.size(); k++) values(begin_ + k) = tmp[k];
  }
};

}  // namespace Kokkos
