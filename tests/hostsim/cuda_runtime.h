// Host compilation of the emitted per-mechanism device headers (TEST
// INFRASTRUCTURE ONLY: tests/test_emitted_host.py).  It stands in for
// <cuda_runtime.h>: the CUDA function qualifiers become plain C++, and the
// few warp intrinsics the headers use become their one-thread meaning.
// The emitted arithmetic itself is unchanged; compiled with
// -ffp-contract=off only its explicit fma() calls fuse, as on the GPU
// (built with --fmad=false).
#pragma once
// System headers first: glibc uses the token __noinline__ in attributes.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <math.h>
#include <stdint.h>
#include <type_traits>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))

using std::isfinite;

template <class T>
inline T __ldg(const T* p) { return *p; }
inline void __syncwarp(unsigned = 0xffffffffu) {}
template <class T>
inline T __shfl_sync(unsigned, T v, int, int = 32) { return v; }
inline int __any_sync(unsigned, int p) { return p; }
inline int __all_sync(unsigned, int p) { return p; }
inline long long __double_as_longlong(double x) {
  long long r;
  std::memcpy(&r, &x, sizeof r);
  return r;
}
inline double __longlong_as_double(long long x) {
  double r;
  std::memcpy(&r, &x, sizeof r);
  return r;
}
