// Device-side vocabulary shared by every generated mechanism header and the
// solver kernels: per-cell status codes, strided accessors over the
// cell-innermost (LayoutLeft) arrays, and math constants used by the emitted
// rate-constant expressions.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#ifndef M_LN10
#define M_LN10 2.30258509299404568402
#endif

namespace mkpp {

// Per-cell outcome codes; values follow mkpp_host::CellErrorCode
// (src/mkpp_host/include/mkpp_host/dispatcher.hpp:15-21).
enum CellStatus : int {
  CELL_SUCCESS = 0,
  CELL_ERR_SINGULAR_MATRIX = 1,
  CELL_ERR_NON_FINITE_STATE = 2,
  CELL_ERR_CONVERGENCE_FAILURE = 3,
  CELL_ERR_NUMERICAL_FAILURE = 4,
  CELL_ERR_CHECKPOINT_OVERFLOW = 5,   // more accepted steps than checkpoint slots
};

// Read-only strided view of one cell's row in a LayoutLeft (cells x n) array:
// element s of cell c lives at base[c + ncells * s].
struct CellRow {
  const double* __restrict__ base;
  size_t stride;
  __device__ __forceinline__ double operator()(int s) const { return __ldg(base + (size_t)s * stride); }
};

// Writable strided row (used for the rate-constant table).
struct CellRowOut {
  double* __restrict__ base;
  size_t stride;
  __device__ __forceinline__ void set(int r, double v) const { base[(size_t)r * stride] = v; }
};

// Rate constants read back from the (reactions x cells) table.
struct KTable {
  const double* __restrict__ base;
  size_t stride;
  __device__ __forceinline__ double operator()(int r) const { return __ldg(base + (size_t)r * stride); }
};

// Rate constants held in a private array (adjoint / small mechanisms).
template <int N>
struct KLocal {
  double v[N];
  __device__ __forceinline__ double operator()(int r) const { return v[r]; }
  __device__ __forceinline__ void set(int r, double x) { v[r] = x; }
};

__device__ __forceinline__ bool finite(double x) { return isfinite(x); }

}  // namespace mkpp
