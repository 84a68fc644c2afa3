// Minimal host-only stand-in for the subset of the Kokkos API that the
// MaHyCo reference sources use.  It exists only so that the unmodified
// reference can be compiled here as a CPU oracle (test infrastructure; never
// linked into the product).
//
// Subset covered (by grep over the reference sources):
//   View<T*>, View<T**>, View<T***>, View<T> with operator(), 1-D operator[],
//   data(), handle-copy semantics (std::swap swaps buffers), deep_copy,
//   parallel_for(n | label,n, f), parallel_reduce(n | label,n, f, reducer)
//   with Sum / Min / Max / any user reducer exposing init/join/reference,
//   initialize / finalize, hwloc queries, impl_max_hardware_threads.
//
// Every allocation carries a zero-filled front guard of kGuard elements.  The
// reference reads index (size_t)-1 at boundary nodes (remap/DualPhaseRemap1.cc
// :52-57, DualPhaseRemap2.cc:56-61) and only multiplies the value by a zero
// mass flux; under real Kokkos that read lands in the allocation header, here
// it lands in zeros.
#ifndef ORACLE_KOKKOS_SHIM_CORE_HPP
#define ORACLE_KOKKOS_SHIM_CORE_HPP

#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <functional>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KOKKOS_LAMBDA [=]
#define KOKKOS_INLINE_FUNCTION inline

namespace Kokkos {

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}

struct LayoutLeft {};
struct LayoutRight {};

struct OpenMP {
  static int impl_max_hardware_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
  }
};
using DefaultExecutionSpace = OpenMP;

namespace hwloc {
inline bool available() { return false; }
inline unsigned get_available_numa_count() { return 1; }
inline unsigned get_available_cores_per_numa() { return 1; }
inline unsigned get_available_threads_per_core() { return 1; }
}  // namespace hwloc

namespace shim_detail {
constexpr std::size_t kGuard = 64;

template <class T>
struct Storage {
  std::vector<T> buf;
  T* base = nullptr;
  explicit Storage(std::size_t n) : buf(n + kGuard, T()) {
    for (auto& x : buf) x = zero_of<T>();
    base = buf.data() + kGuard;
  }
  template <class U>
  static U zero_of() {
    U u;
    zero_fill(u);
    return u;
  }
  template <class U>
  static void zero_fill(U& u) {
    if constexpr (std::is_arithmetic_v<U>) {
      u = U(0);
    } else {
      for (auto& e : u) zero_fill(e);
    }
  }
};

template <class T>
struct Rank {
  using value = T;
  static constexpr int r = 0;
};
template <class T>
struct Rank<T*> {
  using value = T;
  static constexpr int r = 1;
};
template <class T>
struct Rank<T**> {
  using value = T;
  static constexpr int r = 2;
};
template <class T>
struct Rank<T***> {
  using value = T;
  static constexpr int r = 3;
};
}  // namespace shim_detail

template <class DataType, class... Props>
class View {
  using R = shim_detail::Rank<DataType>;

 public:
  using value_type = typename R::value;
  static constexpr int rank = R::r;

  View() = default;
  // Rank-0 view wrapping caller memory (used by user reducers' view()).
  explicit View(value_type* p) : unmanaged_(p) {}
  value_type& operator()() const { return *unmanaged_; }
  View(const std::string&, std::size_t n0, std::size_t n1 = 1,
       std::size_t n2 = 1)
      : n0_(n0), n1_(rank >= 2 ? n1 : 1), n2_(rank >= 3 ? n2 : 1) {
    store_ = std::make_shared<shim_detail::Storage<value_type>>(n0_ * n1_ *
                                                                n2_);
  }

  value_type& operator()(std::size_t i) const { return store_->base[i]; }
  value_type& operator()(std::size_t i, std::size_t j) const {
    return store_->base[i * n1_ + j];
  }
  value_type& operator()(std::size_t i, std::size_t j, std::size_t k) const {
    return store_->base[(i * n1_ + j) * n2_ + k];
  }
  value_type& operator[](std::size_t i) const { return store_->base[i]; }
  value_type* data() const { return store_ ? store_->base : unmanaged_; }
  std::size_t extent(int d) const { return d == 0 ? n0_ : d == 1 ? n1_ : n2_; }
  std::size_t size() const { return n0_ * n1_ * n2_; }

 private:
  std::size_t n0_ = 0, n1_ = 1, n2_ = 1;
  std::shared_ptr<shim_detail::Storage<value_type>> store_;
  value_type* unmanaged_ = nullptr;
};

template <class A, class B>
inline void deep_copy(const A& dst, const B& src) {
  const std::size_t n = dst.size();
  for (std::size_t i = 0; i < n; ++i) dst.data()[i] = src.data()[i];
}

// ---- reducers -------------------------------------------------------------
template <class T>
struct Sum {
  using value_type = T;
  T& ref;
  explicit Sum(T& r) : ref(r) {}
  void init(T& v) const { v = T(0); }
  void join(T& dest, const T& src) const { dest += src; }
  T& reference() const { return ref; }
};
template <class T>
struct Min {
  using value_type = T;
  T& ref;
  explicit Min(T& r) : ref(r) {}
  void init(T& v) const { v = std::numeric_limits<T>::max(); }
  void join(T& dest, const T& src) const {
    if (src < dest) dest = src;
  }
  T& reference() const { return ref; }
};
template <class T>
struct Max {
  using value_type = T;
  T& ref;
  explicit Max(T& r) : ref(r) {}
  void init(T& v) const { v = std::numeric_limits<T>::lowest(); }
  void join(T& dest, const T& src) const {
    if (src > dest) dest = src;
  }
  T& reference() const { return ref; }
};

// ---- dispatch -------------------------------------------------------------
template <class F>
inline void parallel_for(std::size_t n, const F& f) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)n; ++i) f((std::size_t)i);
#else
  for (std::size_t i = 0; i < n; ++i) f(i);
#endif
}
template <class F>
inline void parallel_for(const std::string&, std::size_t n, const F& f) {
  parallel_for(n, f);
}

template <class F, class Reducer>
inline void parallel_reduce(std::size_t n, const F& f, const Reducer& red) {
  using T = typename Reducer::value_type;
  T acc;
  red.init(acc);
#ifdef _OPENMP
#pragma omp parallel
  {
    T local;
    red.init(local);
#pragma omp for schedule(static) nowait
    for (long long i = 0; i < (long long)n; ++i) f((std::size_t)i, local);
#pragma omp critical
    red.join(acc, local);
  }
#else
  for (std::size_t i = 0; i < n; ++i) f(i, acc);
#endif
  red.reference() = acc;
}
template <class F, class Reducer>
inline void parallel_reduce(const std::string&, std::size_t n, const F& f,
                            const Reducer& red) {
  parallel_reduce(n, f, red);
}

}  // namespace Kokkos

#endif  // ORACLE_KOKKOS_SHIM_CORE_HPP
