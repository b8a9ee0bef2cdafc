// FP64 FMA throughput probe: the denominator of the FP64 roofline.
//
// Every thread runs 8 independent FMA chains so the FP64 pipe, not the FMA
// latency, bounds the kernel.  FLOPs = 2 * 8 * iters * threads.
#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(256, 1) dfma_chains(double* out, int iters, double b, double c) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
  double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      x0 = fma(x0, b, c); x1 = fma(x1, b, c); x2 = fma(x2, b, c); x3 = fma(x3, b, c);
      x4 = fma(x4, b, c); x5 = fma(x5, b, c); x6 = fma(x6, b, c); x7 = fma(x7, b, c);
    }
  }
  const double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 12345.678) out[blockIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" {

// Launch blocks x threads DFMA chains of `iters` x 4 x 8 FMAs on `stream`.
// Returns the FLOP count of the launch, or -1 on a launch error.
double mkpp_probe_fp64_fma(double* out, int blocks, int threads, int iters, void* stream) {
  dfma_chains<<<blocks, threads, 0, (cudaStream_t)stream>>>(out, iters, 0.999999999, 1e-12);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  return 2.0 * 8.0 * 4.0 * (double)iters * (double)threads * (double)blocks;
}

}  // extern "C"
