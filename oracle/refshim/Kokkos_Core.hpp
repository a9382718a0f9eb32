// Kokkos_Core.hpp — minimal host-only stand-in for the parts of Kokkos 3.5
// that FIESTA's RHS path uses, so that the reference's own kernel sources
// (src/*.hpp, src/cart3d.cpp, src/cart2d.cpp, src/bc.cpp, src/rk.cpp) compile
// unmodified on the CPU as a parity checker.
//
// TEST INFRASTRUCTURE ONLY (used by oracle/ref_build.sh); never shipped.
//
// Kokkos contributes no arithmetic to the path: it dispatches loops and
// takes Max reductions, which is all this file does.  Views are
// reference-counted, zero-initialised host arrays; the default layout is
// LayoutLeft, the layout of the reference's CUDA build.
#ifndef FST_KOKKOS_SHIM_CORE_HPP
#define FST_KOKKOS_SHIM_CORE_HPP

#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <initializer_list>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "Kokkos_Macros.hpp"

namespace Kokkos {

struct LayoutLeft {};
struct LayoutRight {};
struct HostSpace {};
struct DefaultExecutionSpace {
  typedef LayoutLeft array_layout;
};

namespace shim {
template <class T>
struct rank_of {
  static const int value = 0;
  typedef T type;
};
template <class T>
struct rank_of<T*> {
  static const int value = rank_of<T>::value + 1;
  typedef typename rank_of<T>::type type;
};
}  // namespace shim

template <class DataType, class Layout = DefaultExecutionSpace::array_layout>
class View {
 public:
  typedef typename shim::rank_of<DataType>::type value_type;
  static const int Rank = shim::rank_of<DataType>::value;
  typedef View<DataType, Layout> HostMirror;

  View() : ptr_(nullptr) {
    for (int r = 0; r < 8; ++r) ext_[r] = 0, str_[r] = 0;
  }
  explicit View(const std::string& label, size_t n0 = 1, size_t n1 = 1, size_t n2 = 1,
                size_t n3 = 1, size_t n4 = 1, size_t n5 = 1)
      : label_(label) {
    size_t n[6] = {n0, n1, n2, n3, n4, n5};
    for (int r = 0; r < 8; ++r) ext_[r] = 1, str_[r] = 0;
    size_t total = 1;
    for (int r = 0; r < Rank; ++r) ext_[r] = n[r], total *= n[r];
    if (std::is_same<Layout, LayoutLeft>::value) {
      size_t s = 1;
      for (int r = 0; r < Rank; ++r) str_[r] = s, s *= ext_[r];
    } else {
      size_t s = 1;
      for (int r = Rank - 1; r >= 0; --r) str_[r] = s, s *= ext_[r];
    }
    store_ = std::make_shared<std::vector<value_type>>(total, value_type());
    ptr_ = store_->data();
  }

  template <class... I>
  inline value_type& operator()(I... idx) const {
    static_assert(sizeof...(I) == (size_t)Rank, "wrong number of View indices");
    const long long ii[] = {(long long)idx...};
    size_t off = 0;
    for (int r = 0; r < Rank; ++r) off += (size_t)ii[r] * str_[r];
    return ptr_[off];
  }

  size_t extent(int r) const { return ext_[r]; }
  size_t size() const {
    size_t t = 1;
    for (int r = 0; r < Rank; ++r) t *= ext_[r];
    return Rank == 0 ? 0 : t;
  }
  value_type* data() const { return ptr_; }
  const std::string& label() const { return label_; }

 private:
  std::shared_ptr<std::vector<value_type>> store_;
  value_type* ptr_;
  size_t ext_[8];
  size_t str_[8];
  std::string label_;
};

template <class V>
inline V create_mirror_view(const V& v) {
  return v;
}
template <class D, class L>
inline void deep_copy(const View<D, L>& dst, const View<D, L>& src) {
  if (dst.data() == src.data()) return;
  size_t n = dst.size();
  for (size_t q = 0; q < n; ++q) dst.data()[q] = src.data()[q];
}
template <class D, class L>
inline void deep_copy(const View<D, L>& dst, const typename View<D, L>::value_type& val) {
  size_t n = dst.size();
  for (size_t q = 0; q < n; ++q) dst.data()[q] = val;
}

template <int N>
struct Rank {
  static const int value = N;
};

template <class R>
struct MDRangePolicy {
  static const int N = R::value;
  long long b[N], e[N];
  MDRangePolicy() {
    for (int r = 0; r < N; ++r) b[r] = 0, e[r] = 0;
  }
  MDRangePolicy(std::initializer_list<long long> lo, std::initializer_list<long long> hi) {
    int r = 0;
    for (long long x : lo) b[r++] = x;
    r = 0;
    for (long long x : hi) e[r++] = x;
  }
  MDRangePolicy(std::initializer_list<long long> lo, std::initializer_list<long long> hi,
                std::initializer_list<long long> /*tile*/)
      : MDRangePolicy(lo, hi) {}
};

template <class T>
struct Max {
  T& ref;
  explicit Max(T& r) : ref(r) {}
};

namespace shim {
template <class F>
inline void run(const MDRangePolicy<Rank<2>>& p, const F& f) {
#pragma omp parallel for schedule(static)
  for (long long i = p.b[0]; i < p.e[0]; ++i)
    for (long long j = p.b[1]; j < p.e[1]; ++j) f((int)i, (int)j);
}
template <class F>
inline void run(const MDRangePolicy<Rank<3>>& p, const F& f) {
#pragma omp parallel for schedule(static)
  for (long long i = p.b[0]; i < p.e[0]; ++i)
    for (long long j = p.b[1]; j < p.e[1]; ++j)
      for (long long k = p.b[2]; k < p.e[2]; ++k) f((int)i, (int)j, (int)k);
}
template <class F>
inline void run(const MDRangePolicy<Rank<4>>& p, const F& f) {
#pragma omp parallel for schedule(static)
  for (long long i = p.b[0]; i < p.e[0]; ++i)
    for (long long j = p.b[1]; j < p.e[1]; ++j)
      for (long long k = p.b[2]; k < p.e[2]; ++k)
        for (long long l = p.b[3]; l < p.e[3]; ++l) f((int)i, (int)j, (int)k, (int)l);
}
}  // namespace shim

template <class P, class F>
inline void parallel_for(const P& p, const F& f) {
  shim::run(p, f);
}
template <class P, class F>
inline void parallel_for(const std::string&, const P& p, const F& f) {
  shim::run(p, f);
}

// Max reduction; the start value is Kokkos' reduction_identity<T>::max(),
// i.e. the lowest finite T.  Threads reduce static chunks of the outer
// index and join with Kokkos' Max join (`if (src > dst) dst = src`, which
// never takes a NaN), so the result is the serial maximum.
template <class F, class T>
inline void parallel_reduce(const MDRangePolicy<Rank<2>>& p, const F& f, Max<T> m) {
  T g = std::numeric_limits<T>::lowest();
#pragma omp parallel
  {
    T l = std::numeric_limits<T>::lowest();
#pragma omp for schedule(static)
    for (long long i = p.b[0]; i < p.e[0]; ++i)
      for (long long j = p.b[1]; j < p.e[1]; ++j) f((int)i, (int)j, l);
#pragma omp critical(fst_shim_max)
    if (l > g) g = l;
  }
  m.ref = g;
}
template <class F, class T>
inline void parallel_reduce(const MDRangePolicy<Rank<3>>& p, const F& f, Max<T> m) {
  T g = std::numeric_limits<T>::lowest();
#pragma omp parallel
  {
    T l = std::numeric_limits<T>::lowest();
#pragma omp for schedule(static)
    for (long long i = p.b[0]; i < p.e[0]; ++i)
      for (long long j = p.b[1]; j < p.e[1]; ++j)
        for (long long k = p.b[2]; k < p.e[2]; ++k) f((int)i, (int)j, (int)k, l);
#pragma omp critical(fst_shim_max)
    if (l > g) g = l;
  }
  m.ref = g;
}

inline void fence() {}

struct InitArguments {
  int ndevices = 1;
  int num_threads = -1;
};
inline void initialize(const InitArguments&) {}
inline void initialize(int&, char**) {}
inline void finalize() {}

namespace Profiling {
inline void pushRegion(const std::string&) {}
inline void popRegion() {}
}  // namespace Profiling

}  // namespace Kokkos

#endif
