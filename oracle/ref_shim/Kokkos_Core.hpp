// TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// Minimal single-threaded stand-in for the part of Kokkos 5.1.1 that the reference's
// groundwater sources use (src/re/ReSolver.cpp, src/re/VanGenuchten.hpp, src/re/GwFields.hpp,
// src/linear/DomainDecomposition.cpp, src/core/MpiComm.cpp, include/frehg2/core/*.hpp), so
// those files compile here unchanged into oracle/_ref.  Kokkos is not installed in this image.
//
// Semantics kept from Kokkos: a View is a reference-counted handle (copies alias the same
// storage) whose managed allocations start zero-filled; parallel_for over a range or an
// MDRange calls the functor once per index (the reference only converts loops whose
// iterations write disjoint cells, include/frehg2/core/ParallelFor.hpp:3-10, so a serial
// order gives the same bits); the math functions are the C library's.  Host and "device"
// memory spaces are one space, so create_mirror_view returns the view itself.
#ifndef FREHG_REF_SHIM_KOKKOS_CORE_HPP
#define FREHG_REF_SHIM_KOKKOS_CORE_HPP

#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]

namespace Kokkos {

struct LayoutRight {};
struct LayoutLeft {};
struct HostSpace {
  using memory_space = HostSpace;
};
struct Serial {
  using memory_space = HostSpace;
  using execution_space = Serial;
};
using DefaultExecutionSpace = Serial;
using DefaultHostExecutionSpace = Serial;

enum MemoryTraitsFlags : unsigned { Unmanaged = 1u };
template <unsigned Flags>
struct MemoryTraits {};

template <class DataType, class... Props>
class View;

// One-dimensional view (the only rank the groundwater path instantiates).
template <class T, class... Props>
class View<T*, Props...> {
 public:
  using value_type = T;
  using non_const_value_type = std::remove_const_t<T>;

  View() = default;
  View(const std::string& label, std::size_t n)
      : store_(new non_const_value_type[n](), std::default_delete<non_const_value_type[]>()),
        ptr_(store_.get()),
        n_(n),
        label_(label) {}
  View(T* ptr, std::size_t n) : ptr_(ptr), n_(n) {}  // unmanaged wrap

  template <class U, class... P2,
            class = std::enable_if_t<std::is_convertible_v<U*, T*>>>
  View(const View<U*, P2...>& o)  // NOLINT: implicit like Kokkos' compatible-view copy
      : store_(o.store_), ptr_(o.ptr_), n_(o.n_), label_(o.label_) {}

  T& operator()(std::size_t i) const { return ptr_[i]; }
  T& operator[](std::size_t i) const { return ptr_[i]; }
  T* data() const { return ptr_; }
  std::size_t extent(int) const { return n_; }
  std::size_t size() const { return n_; }
  std::size_t span() const { return n_; }
  const std::string& label() const { return label_; }
  bool is_allocated() const { return ptr_ != nullptr; }

 private:
  template <class, class...>
  friend class View;
  std::shared_ptr<non_const_value_type> store_;
  T* ptr_ = nullptr;
  std::size_t n_ = 0;
  std::string label_;
};

template <class V>
inline V create_mirror_view(const V& v) {
  return v;
}

template <class T1, class... P1, class T2, class... P2>
inline void deep_copy(const View<T1*, P1...>& dst, const View<T2*, P2...>& src) {
  if (static_cast<const void*>(dst.data()) == static_cast<const void*>(src.data())) return;
  const std::size_t n = dst.size() < src.size() ? dst.size() : src.size();
  for (std::size_t i = 0; i < n; ++i) dst(i) = src(i);
}

template <class T1, class... P1>
inline void deep_copy(const View<T1*, P1...>& dst, const std::remove_const_t<T1>& value) {
  for (std::size_t i = 0; i < dst.size(); ++i) dst(i) = value;
}

template <class Exec = Serial>
struct RangePolicy {
  RangePolicy(long b, long e) : begin(b), end(e) {}
  long begin, end;
};

template <unsigned N>
struct Rank {
  static constexpr unsigned rank = N;
};

template <class Exec, class R>
struct MDRangePolicy {
  MDRangePolicy(std::initializer_list<long> b, std::initializer_list<long> e) {
    unsigned d = 0;
    for (long v : b) lo[d++] = v;
    d = 0;
    for (long v : e) hi[d++] = v;
  }
  long lo[3] = {0, 0, 0};
  long hi[3] = {0, 0, 0};
};

template <class Exec, class F>
inline void parallel_for(const char*, const RangePolicy<Exec>& p, const F& f) {
  for (long i = p.begin; i < p.end; ++i) f(static_cast<int>(i));
}

template <class F>
inline void parallel_for(const char* name, long n, const F& f) {
  parallel_for(name, RangePolicy<Serial>(0, n), f);
}

template <class Exec, class F>
inline void parallel_for(const char*, const MDRangePolicy<Exec, Rank<2>>& p, const F& f) {
  for (long i = p.lo[0]; i < p.hi[0]; ++i)
    for (long j = p.lo[1]; j < p.hi[1]; ++j) f(static_cast<int>(i), static_cast<int>(j));
}

template <class Exec, class F>
inline void parallel_for(const char*, const MDRangePolicy<Exec, Rank<3>>& p, const F& f) {
  for (long i = p.lo[0]; i < p.hi[0]; ++i)
    for (long j = p.lo[1]; j < p.hi[1]; ++j)
      for (long k = p.lo[2]; k < p.hi[2]; ++k)
        f(static_cast<int>(i), static_cast<int>(j), static_cast<int>(k));
}

class Timer {
 public:
  Timer() : t0_(std::chrono::steady_clock::now()) {}
  double seconds() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
  }
  void reset() { t0_ = std::chrono::steady_clock::now(); }

 private:
  std::chrono::steady_clock::time_point t0_;
};

namespace Profiling {
inline void pushRegion(const std::string&) {}
inline void popRegion() {}
}  // namespace Profiling

using std::exp;
using std::fabs;
using std::fmax;
using std::fmin;
using std::isnan;
using std::log;
using std::pow;
using std::sqrt;

inline void initialize(int = 0, char** = nullptr) {}
inline void finalize() {}

}  // namespace Kokkos

#endif  // FREHG_REF_SHIM_KOKKOS_CORE_HPP
