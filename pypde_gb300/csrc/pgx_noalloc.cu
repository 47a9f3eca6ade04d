// Zero-allocation variant of pgx_cheb_transform_2d.
//
// Some callers cannot let a library allocate device memory: host codes that
// own every byte of device memory through their own pool or a fixed budget,
// and time loops that must not hit the implicit device-wide synchronisation
// of cudaMalloc / cudaFree.  pgx_cheb_transform_2d needs scratch between its
// two axis passes (and, on first use of a length, device twiddle tables); this
// entry point takes both from file-scope static device arrays instead, so it
// calls no cudaMalloc, cudaFree or other allocating routine.
//
// Every GPU that loads the library holds these arrays until the process exits.
// All calls on a device share them, and they keep the last call's contents:
// calls that overlap on the GPU (different streams, or host threads racing)
// race on the scratch.  Nothing here has to start at zero: each call rewrites
// the twiddle tables and every scratch element it later reads.

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "pgx.h"

// Defined in pgx_api.cu: one DCT-I pass along an axis with a given table.
int pgx_dct_pass(const double* in, int64_t in_s0, int64_t in_s1, int32_t n_in, double* out, int64_t out_s0,
                 int64_t out_s1, int32_t n_out, int32_t n, int32_t nlines, int32_t axis, int32_t mode,
                 const double* tab, bool fft, void* stream);
bool pgx_fft_length_ok(int n);

namespace {

// complex entries per table: 2(n-1) twiddles and (n-1) / 2 for the n-1 fold coefficients, for every allowed n
constexpr int kTwiddles = 3 * PGX_LMAX;

static __device__ __align__(256) double g_noalloc_scratch[PGX_NOALLOC_SCRATCH_DOUBLES];
static __device__ __align__(256) double2 g_noalloc_twiddles[2 * kTwiddles];

// exp(-2 pi i k / L) for both axes' lengths, exact on the axes of the unit circle, each table
// followed by the fold coefficients 0.5 + Im(tw[k]) = 1/2 - sin(2 pi k / L) (k < L / 2).
__global__ void noalloc_fill_twiddles(int L0, int L1) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < L0 + L1; i += gridDim.x * blockDim.x) {
    const int table = i < L0 ? 0 : 1;
    const int k = table ? i - L0 : i;
    const int L = table ? L1 : L0;
    double s, c;
    sincospi(2.0 * (double)k / (double)L, &s, &c);
    if ((4 * k) % L == 0) {
      const int q = (4 * k) / L;
      c = q == 0 ? 1.0 : (q == 2 ? -1.0 : 0.0);
      s = q == 1 ? 1.0 : (q == 3 ? -1.0 : 0.0);
    }
    g_noalloc_twiddles[table * kTwiddles + k] = make_double2(c, -s);
    if (k < L / 2) reinterpret_cast<double*>(g_noalloc_twiddles + table * kTwiddles + L)[k] = 0.5 + (-s);
  }
}

struct DeviceArrays {
  double* scratch = nullptr;
  double2* twiddles = nullptr;
  bool ready = false;
};
constexpr int kMaxDevices = 64;
DeviceArrays g_arrays[kMaxDevices];
std::mutex g_setup_mu;

// Device addresses of the static arrays for the current device, looked up once
// per device (host code only sees host-side stand-ins for the symbols).
int device_arrays(DeviceArrays** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return PGX_E_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return PGX_E_ARG;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  DeviceArrays& d = g_arrays[dev];
  if (!d.ready) {
    e = cudaGetSymbolAddress((void**)&d.scratch, g_noalloc_scratch);
    if (e != cudaSuccess) return PGX_E_CUDA;
    e = cudaGetSymbolAddress((void**)&d.twiddles, g_noalloc_twiddles);
    if (e != cudaSuccess) return PGX_E_CUDA;
    d.ready = true;
  }
  *out = &d;
  return PGX_OK;
}

}  // namespace

extern "C" int pgx_cheb_transform_2d_noalloc(const double* in, int64_t in_s0, int64_t in_s1, int32_t n0_in,
                                             int32_t n1_in, double* out, int64_t out_s0, int64_t out_s1,
                                             int32_t n0_out, int32_t n1_out, int32_t N0, int32_t N1, int32_t mode,
                                             void* stream) {
  if (!in || !out || mode < 0 || mode > 2 || N0 < 2 || N1 < 2 || N0 > PGX_LMAX - 8 || N1 > PGX_LMAX - 8 ||
      n0_in < 0 || n0_in > N0 || n1_in < 0 || n1_in > N1 || n0_out < 0 || n0_out > N0 || n1_out < 0 ||
      n1_out > N1)
    return PGX_E_ARG;
  // the dense fallback of other lengths would need an N x N table: only FFT lengths here
  if (!pgx_fft_length_ok(N0) || !pgx_fft_length_ok(N1)) return PGX_E_ARG;
  if ((int64_t)n0_out * n1_in > (int64_t)PGX_NOALLOC_SCRATCH_DOUBLES) return PGX_E_ARG;
  DeviceArrays* d = nullptr;
  int rc = device_arrays(&d);
  if (rc) return rc;
  const int L0 = 2 * (N0 - 1), L1 = 2 * (N1 - 1);
  cudaStream_t s = (cudaStream_t)stream;
  noalloc_fill_twiddles<<<(L0 + L1 + 255) / 256, 256, 0, s>>>(L0, L1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return PGX_E_CUDA;
  const double* tw0 = reinterpret_cast<const double*>(d->twiddles);
  const double* tw1 = reinterpret_cast<const double*>(d->twiddles + kTwiddles);
  rc = pgx_dct_pass(in, in_s0, in_s1, n0_in, d->scratch, n1_in, 1, n0_out, N0, n1_in, 0, mode, tw0, true, stream);
  if (rc) return rc;
  return pgx_dct_pass(d->scratch, n1_in, 1, n1_in, out, out_s0, out_s1, n1_out, N1, n0_out, 1, mode, tw1, true,
                      stream);
}
