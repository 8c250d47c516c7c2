// Kokkos_Core.hpp -- a serial stand-in for the part of the Kokkos API that
// the reference's deduplicators use, so that their own sources
// (src/{tree,list,basic}_approach.cpp) compile and run on the host.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build.py into oracle/_ref/ and
// used by tests to compare the oracle's restatement with the reference code.
// It fixes the semantics the reference leaves to Kokkos, as a Serial
// execution space would: every parallel loop runs its indices in ascending
// order (team loops: league rank, then team rank, then the team's strided
// share of a TeamThreadRange), scans run once with `final` set, atomics are
// plain operations.  Views are shallow handles, like Kokkos Views.
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <type_traits>
#include <functional>
#include <fstream>
#include <iostream>
#include <map>
#include <set>
#include <unordered_map>
#include <utility>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [=, *this]

namespace Kokkos {

struct Serial {
  static void fence() {}
};
using DefaultExecutionSpace = Serial;
using DefaultHostExecutionSpace = Serial;
struct HostSpace {};
template <unsigned T>
struct MemoryTraits {};
enum : unsigned { Unmanaged = 1, RandomAccess = 2, Atomic = 4 };
struct ALL_t {};
constexpr ALL_t ALL{};
// Kokkos::AUTO and Kokkos::AUTO(): a serial team has one member
struct AUTO_t {
  constexpr AUTO_t operator()() const { return *this; }
  constexpr operator int() const { return 1; }
};
constexpr AUTO_t AUTO{};

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}
inline void fence() {}
inline void fence(const std::string&) {}

namespace Profiling {
inline void pushRegion(const std::string&) {}
inline void popRegion() {}
}  // namespace Profiling

// ---- Views ------------------------------------------------------------------
template <class D>
struct ViewTraits;
template <class T>
struct ViewTraits<T*> {
  using value_type = T;
  static constexpr size_t static_extent = 0;
};
template <class T, size_t N>
struct ViewTraits<T[N]> {
  using value_type = T;
  static constexpr size_t static_extent = N;
};

template <class DataType, class... Props>
class View {
 public:
  using traits = ViewTraits<DataType>;
  using value_type = typename traits::value_type;
  using non_const_value_type = typename std::remove_const<value_type>::type;
  using HostMirror = View<DataType, Props...>;
  using size_type = size_t;

  View() = default;
  explicit View(const std::string& label, size_t n = traits::static_extent) : label_(label) { alloc(n); }
  View(const char* label, size_t n = traits::static_extent) : label_(label) { alloc(n); }
  View(value_type* p, size_t n) : ptr_(p), n_(n) {}
  template <class... Q>
  View(const View<DataType, Q...>& o) : owner_(o.owner_), ptr_(o.ptr_), n_(o.n_), label_(o.label_) {}

  value_type& operator()(size_t i) const { return ptr_[i]; }
  value_type& operator[](size_t i) const { return ptr_[i]; }
  value_type* data() const { return ptr_; }
  size_t extent(int d) const { return d == 0 ? n_ : 1; }
  size_t extent_int(int d) const { return extent(d); }
  size_t size() const { return n_; }
  size_t span() const { return n_; }
  const std::string& label() const { return label_; }
  bool is_allocated() const { return ptr_ != nullptr; }

  void alloc(size_t n) {
    owner_ = std::shared_ptr<non_const_value_type>(new non_const_value_type[n ? n : 1](),
                                                   std::default_delete<non_const_value_type[]>());
    ptr_ = owner_.get();
    n_ = n;
  }

  std::shared_ptr<non_const_value_type> owner_;
  value_type* ptr_ = nullptr;
  size_t n_ = 0;
  std::string label_;
};

template <class V>
V create_mirror_view(const V& v) {
  return v;
}
template <class S, class V>
V create_mirror_view(const S&, const V& v) {
  return v;
}
template <class V>
V create_mirror(const V& v) {
  V m(v.label(), v.size());
  std::copy(v.data(), v.data() + v.size(), m.data());
  return m;
}

template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...>& dst, const View<D2, P2...>& src) {
  const size_t n = std::min(dst.size(), src.size());
  if (n && dst.data() != src.data()) std::memmove(dst.data(), src.data(), n * sizeof(*dst.data()));
}
template <class D, class... P, class T>
typename std::enable_if<!std::is_class<T>::value || std::is_same<T, typename View<D, P...>::value_type>::value>::type
deep_copy(const View<D, P...>& dst, const T& value) {
  for (size_t i = 0; i < dst.size(); i++) dst(i) = value;
}
template <class E, class V1, class V2>
void deep_copy(const E&, const V1& dst, const V2& src) {
  deep_copy(dst, src);
}

template <class D, class... P>
View<D, P...> subview(const View<D, P...>& v, std::pair<size_t, size_t> r) {
  View<D, P...> s;
  s.owner_ = v.owner_;
  s.ptr_ = v.ptr_ + r.first;
  s.n_ = r.second - r.first;
  s.label_ = v.label_;
  return s;
}
template <class D, class... P, class A, class B>
View<D, P...> subview(const View<D, P...>& v, std::pair<A, B> r) {
  return subview(v, std::pair<size_t, size_t>((size_t)r.first, (size_t)r.second));
}
template <class D, class... P>
View<D, P...> subview(const View<D, P...>& v, ALL_t) {
  return v;
}

template <class D, class... P>
void resize(View<D, P...>& v, size_t n) {
  if (v.size() == n && v.data()) return;  // same extent: the view is kept
  View<D, P...> w(v.label(), n);
  const size_t m = std::min(n, v.size());
  if (m) std::memcpy(w.data(), v.data(), m * sizeof(*v.data()));
  v = w;
}
template <class D, class... P>
void realloc(View<D, P...>& v, size_t n) {
  v = View<D, P...>(v.label(), n);
}

// ---- atomics ------------------------------------------------------------------
template <class T, class U>
T atomic_fetch_add(T* p, U v) {
  T o = *p;
  *p = o + (T)v;
  return o;
}
template <class T, class U>
void atomic_add(T* p, U v) {
  *p = *p + (T)v;
}
template <class T, class U>
T atomic_add_fetch(T* p, U v) {
  *p = *p + (T)v;
  return *p;
}
template <class T, class U>
T atomic_fetch_sub(T* p, U v) {
  T o = *p;
  *p = o - (T)v;
  return o;
}
template <class T, class U>
void atomic_min(T* p, U v) {
  if ((T)v < *p) *p = (T)v;
}
template <class T, class U>
void atomic_max(T* p, U v) {
  if ((T)v > *p) *p = (T)v;
}
template <class T, class U>
T atomic_fetch_max(T* p, U v) {
  T o = *p;
  if ((T)v > o) *p = (T)v;
  return o;
}
template <class T, class U>
T atomic_fetch_min(T* p, U v) {
  T o = *p;
  if ((T)v < o) *p = (T)v;
  return o;
}
template <class T, class U, class W>
T atomic_compare_exchange(T* p, U expected, W desired) {
  T o = *p;
  if (o == (T)expected) *p = (T)desired;
  return o;
}

// ---- execution policies ----------------------------------------------------------
template <class... P>
struct RangePolicy {
  uint64_t b = 0, e = 0;
  RangePolicy(uint64_t b_, uint64_t e_) : b(b_), e(e_) {}
  template <class S>
  RangePolicy(const S&, uint64_t b_, uint64_t e_) : b(b_), e(e_) {}
};

struct TeamMember {
  int league, team, team_sz, league_sz;
  int league_rank() const { return league; }
  int team_rank() const { return team; }
  int team_size() const { return team_sz; }
  int league_size() const { return league_sz; }
  void team_barrier() const {}
  template <class T>
  void team_broadcast(T&, int) const {}
  template <class S>
  S& team_scratch(int) const;
};

template <class... P>
struct TeamPolicy {
  using member_type = TeamMember;
  int league = 0, team = 1;
  TeamPolicy(int l, int t) : league(l), team(t) {}
  TeamPolicy(int l, AUTO_t) : league(l), team(1) {}
  template <class S>
  TeamPolicy(const S&, int l, int t) : league(l), team(t) {}
};

struct TeamThreadRangeT {
  const TeamMember* m;
  uint64_t b, e;
};
inline TeamThreadRangeT TeamThreadRange(const TeamMember& m, uint64_t n) { return {&m, 0, n}; }
inline TeamThreadRangeT TeamThreadRange(const TeamMember& m, uint64_t b, uint64_t e) { return {&m, b, e}; }

namespace Impl {
template <class F>
void range_for(uint64_t b, uint64_t e, const F& f) {
  for (uint64_t i = b; i < e; i++) f(i);
}
}  // namespace Impl

template <class F>
void parallel_for(const TeamThreadRangeT& r, const F& f) {
  // this member's strided share of the range
  for (uint64_t i = r.b + r.m->team; i < r.e; i += r.m->team_sz) f(i);
}
template <class... P, class F>
void parallel_for(const RangePolicy<P...>& p, const F& f) {
  Impl::range_for(p.b, p.e, f);
}
template <class... P, class F>
void parallel_for(const TeamPolicy<P...>& p, const F& f) {
  for (int l = 0; l < p.league; l++)
    for (int t = 0; t < p.team; t++) f(TeamMember{l, t, p.team, p.league});
}
template <class N, class F>
typename std::enable_if<std::is_integral<N>::value>::type parallel_for(N n, const F& f) {
  Impl::range_for(0, (uint64_t)n, f);
}
template <class Pol, class F>
void parallel_for(const std::string&, const Pol& p, const F& f) {
  parallel_for(p, f);
}
template <class Pol, class F>
void parallel_for(const char*, const Pol& p, const F& f) {
  parallel_for(p, f);
}

namespace Impl {
// the type of a functor's second argument (the reduction / scan value)
template <class F>
struct second_arg : second_arg<decltype(&F::operator())> {};
template <class C, class R, class A0, class A1>
struct second_arg<R (C::*)(A0, A1) const> {
  using type = typename std::remove_cv<typename std::remove_reference<A1>::type>::type;
};
template <class C, class R, class A0, class A1, class A2>
struct second_arg<R (C::*)(A0, A1, A2) const> {
  using type = typename std::remove_cv<typename std::remove_reference<A1>::type>::type;
};
}  // namespace Impl

// reductions: only Max and plain sums are used
template <class T>
struct Max {
  T& ref;
  explicit Max(T& r) : ref(r) {}
};
template <class T>
struct Sum {
  T& ref;
  explicit Sum(T& r) : ref(r) {}
};
namespace Impl {
inline void policy_range(uint64_t n, uint64_t& b, uint64_t& e) { b = 0; e = n; }
template <class... P>
void policy_range(const RangePolicy<P...>& p, uint64_t& b, uint64_t& e) { b = p.b; e = p.e; }
}  // namespace Impl
template <class Pol, class F, class T>
void parallel_reduce(const Pol& p, const F& f, Max<T> r) {
  uint64_t b, e;
  Impl::policy_range(p, b, e);
  T acc = std::numeric_limits<T>::lowest();
  for (uint64_t i = b; i < e; i++) f(i, acc);
  r.ref = acc;
}
template <class Pol, class F, class T>
typename std::enable_if<std::is_arithmetic<T>::value>::type parallel_reduce(const Pol& p, const F& f, T& result) {
  uint64_t b, e;
  Impl::policy_range(p, b, e);
  typename Impl::second_arg<F>::type acc = 0;
  for (uint64_t i = b; i < e; i++) f(i, acc);
  result = (T)acc;
}
template <class Pol, class F, class R>
void parallel_reduce(const std::string&, const Pol& p, const F& f, R&& r) {
  parallel_reduce(p, f, std::forward<R>(r));
}

// scans: one pass, `final` set
template <class Pol, class F>
void parallel_scan(const Pol& p, const F& f) {
  uint64_t b, e;
  Impl::policy_range(p, b, e);
  typename Impl::second_arg<F>::type upd = 0;
  for (uint64_t i = b; i < e; i++) f(i, upd, true);
}
template <class Pol, class F, class T>
void parallel_scan(const Pol& p, const F& f, T& total) {
  uint64_t b, e;
  Impl::policy_range(p, b, e);
  typename Impl::second_arg<F>::type upd = 0;
  for (uint64_t i = b; i < e; i++) f(i, upd, true);
  total = (T)upd;
}
template <class Pol, class F>
void parallel_scan(const std::string&, const Pol& p, const F& f) {
  parallel_scan(p, f);
}
template <class Pol, class F, class T>
void parallel_scan(const std::string&, const Pol& p, const F& f, T& total) {
  parallel_scan(p, f, total);
}

struct Timer {
  double seconds() const { return 0; }
  void reset() {}
};

}  // namespace Kokkos
