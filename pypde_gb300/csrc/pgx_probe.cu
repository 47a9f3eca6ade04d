// FP64 fused multiply-add throughput of the GPU, measured in the caller's process.
//
// Every kernel of the time-step path is bound by FP64 instruction issue, not by
// HBM (its arithmetic intensity is far above the FP64 ridge point), so the
// roofline denominator is the rate at which this GPU retires DFMA, at the
// clock it runs at right now.  The benchmark times this kernel with CUDA events
// next to its own timed region, so a different clock bin moves the peak and the
// measured kernels together.
//
// Each thread runs CHAINS independent FMA chains (enough to cover the DFMA
// latency with a few warps per sub-partition); a and b are runtime values so
// nothing folds, and every chain's result is stored.

#include <cuda_runtime.h>
#include <stdint.h>

#include "pgx.h"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(1024) fp64_fma_rate(double* __restrict__ out, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 1e-3 * threadIdx.x + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int64_t pgx_fp64_fma_probe_flops(int32_t ctas, int32_t threads, int32_t iters) {
  return 2ll * kChains * ctas * threads * (int64_t)iters;
}

extern "C" int pgx_fp64_fma_probe(double* out, int32_t ctas, int32_t threads, int32_t iters, void* stream) {
  if (!out || ctas < 1 || threads < 32 || threads > 1024 || (threads & 31) || iters < 1) return PGX_E_ARG;
  fp64_fma_rate<<<ctas, threads, 0, (cudaStream_t)stream>>>(out, iters, 1.0 + 1e-12, 1e-9);
  return cudaGetLastError() == cudaSuccess ? PGX_OK : PGX_E_CUDA;
}
