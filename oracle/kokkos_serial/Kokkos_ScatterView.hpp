// Kokkos_ScatterView.hpp -- serial stand-in (test infrastructure; see
// Kokkos_Core.hpp): a ScatterView is its View; contributions are plain adds.
#pragma once
#include "Kokkos_Core.hpp"

namespace Kokkos {
namespace Experimental {
template <class DataType, class... P>
class ScatterView {
 public:
  View<DataType> v;
  ScatterView() = default;
  template <class V>
  ScatterView(const V& view) : v(view) {}
  View<DataType> access() const { return v; }
  void reset() const {}
  template <class V>
  void reset_except(const V&) const {}
};
template <class V, class S>
void contribute(V&, const S&) {}
}  // namespace Experimental
}  // namespace Kokkos
