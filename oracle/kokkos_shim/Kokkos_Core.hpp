// Minimal host-only stand-in for the Kokkos API surface that MKPP's generated
// solver headers use (TEST AND CPU-BASELINE INFRASTRUCTURE ONLY; no Kokkos exists
// on this image).  It provides:
//   * View<DataType, Props...> for rank 1 and 2 over caller memory, with
//     LayoutLeft / LayoutRight / LayoutStride strides, data(), stride(),
//     extent() and operator();
//   * HostSpace, the math forwarding to <cmath> the generated code calls
//     (exp log pow cbrt sqrt fabs fmax fmin min isfinite);
//   * the KOKKOS_* function macros and KOKKOS_VERSION.
// Loops and parallel dispatch are not provided: oracle/ref_driver.cpp runs
// the per-cell integrate() itself under OpenMP.
#pragma once
#include <cmath>
#include <cstddef>
#include <type_traits>

#define KOKKOS_VERSION 50101
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_DEFAULTED_FUNCTION

namespace Kokkos {

struct LayoutLeft {};
struct LayoutRight {};
struct LayoutStride {};
struct HostSpace {
  using memory_space = HostSpace;
};
struct MemoryUnmanaged {};

namespace shim {
template <class T>
struct rank_of;
template <class T>
struct rank_of<T*> {
  static constexpr unsigned value = 1;
  using elem = T;
};
template <class T>
struct rank_of<T**> {
  static constexpr unsigned value = 2;
  using elem = T;
};
template <class... P>
struct layout_of {
  using type = LayoutRight;
};
template <class... P>
struct layout_of<LayoutLeft, P...> {
  using type = LayoutLeft;
};
template <class... P>
struct layout_of<LayoutStride, P...> {
  using type = LayoutStride;
};
template <class H, class... P>
struct layout_of<H, P...> : layout_of<P...> {};
}  // namespace shim

template <class DataType, class... Props>
class View {
 public:
  using value_type = typename shim::rank_of<DataType>::elem;
  using pointer_type = value_type*;
  using array_layout = typename shim::layout_of<Props...>::type;
  using memory_space = HostSpace;
  static constexpr unsigned rank = shim::rank_of<DataType>::value;

  View() = default;
  // rank 1: contiguous, or strided (LayoutStride)
  View(pointer_type p, std::size_t n0, std::size_t s0 = 1) : p_(p), n0_(n0), s0_(s0) {}
  // rank 2 with explicit strides
  View(pointer_type p, std::size_t n0, std::size_t n1, std::size_t s0, std::size_t s1)
      : p_(p), n0_(n0), n1_(n1), s0_(s0), s1_(s1) {}
  // const-relaxing copy
  template <class D2, class... P2>
  View(const View<D2, P2...>& o) : p_(o.data()), n0_(o.extent(0)), n1_(o.extent(1)), s0_(o.stride(0)), s1_(o.stride(1)) {}

  value_type& operator()(std::size_t i) const { return p_[i * s0_]; }
  value_type& operator()(std::size_t i, std::size_t j) const { return p_[i * s0_ + j * s1_]; }
  value_type& operator[](std::size_t i) const { return p_[i * s0_]; }
  pointer_type data() const { return p_; }
  std::size_t stride(unsigned r) const { return r == 0 ? s0_ : (r == 1 ? s1_ : 1); }
  std::size_t extent(unsigned r) const { return r == 0 ? n0_ : (r == 1 ? n1_ : 1); }
  std::size_t size() const { return n0_ * n1_; }

 private:
  pointer_type p_ = nullptr;
  std::size_t n0_ = 0, n1_ = 1, s0_ = 1, s1_ = 1;
};

inline double exp(double x) { return std::exp(x); }
inline double log(double x) { return std::log(x); }
inline double pow(double x, double y) { return std::pow(x, y); }
inline double cbrt(double x) { return std::cbrt(x); }
inline double sqrt(double x) { return std::sqrt(x); }
inline double fabs(double x) { return std::fabs(x); }
inline double fmax(double x, double y) { return std::fmax(x, y); }
inline double fmin(double x, double y) { return std::fmin(x, y); }
template <class T>
inline T min(T a, T b) { return b < a ? b : a; }
template <class T>
inline T max(T a, T b) { return a < b ? b : a; }
inline bool isfinite(double x) { return std::isfinite(x); }

}  // namespace Kokkos
