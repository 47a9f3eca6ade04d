// GB300 FP64 probe (not part of the library): DFMA throughput and dependent latency, FP64
// tensor-core (mma.sync m8n8k4 f64) throughput, DFMA and DMMA warps run together (do they share
// the FP64 pipe?), FFMA for reference, stream-launch and CUDA-graph node overhead.  The DFMA
// throughput is the FP64 peak the benchmark's roofline fractions use.
//   nvcc -O3 -gencode arch=compute_103a,code=sm_103a -o fp64_probe pypde_gb300/csrc/fp64_probe.cu && ./fp64_probe
#include <cstdio>
#include <cuda_runtime.h>
#include <mma.h>

#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("ERR %s line %d: %s\n", #x, __LINE__, cudaGetErrorString(e)); return 1; } } while (0)

template <int CHAINS>
__global__ void dfma_tp(double* out, int iters, double a, double b) {
  double x[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) x[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <int CHAINS>
__global__ void ffma_tp(float* out, int iters, float a, float b) {
  float x[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) x[c] = threadIdx.x * 1e-3f + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = fmaf(x[c], a, b);
  }
  float s = 0;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void dmma_tp(double* out, int iters) {
  // mma.sync m8n8k4 f64: A 8x4, B 4x8, C 8x8; per thread a:1 b:1 c:2
  double a = threadIdx.x * 1e-3, b = 1.0 - threadIdx.x * 1e-4;
  double c0[4] = {0, 0, 0, 0}, c1[4] = {0, 0, 0, 0};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(c0[k]), "+d"(c1[k]) : "d"(a), "d"(b));
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = c0[0] + c1[0] + c0[1] + c1[1] + c0[2] + c1[2] + c0[3] + c1[3];
}

__global__ void mixed(double* out, int iters, int mode) {
  const int warp = threadIdx.x >> 5;
  const bool fma_warp = (warp & 1) == 0;
  double r = 0.0;
  if (fma_warp && (mode & 1)) {
    double x[8];
    for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
    const double a = 0.999999, b = 1e-7;
    for (int i = 0; i < iters * 4; ++i) {
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    for (int k = 0; k < 8; ++k) r += x[k];
  } else if (!fma_warp && (mode & 2)) {
    double a = threadIdx.x * 1e-3, b = 1.0 - threadIdx.x * 1e-4;
    double c0[4] = {0, 0, 0, 0}, c1[4] = {0, 0, 0, 0};
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < 4; ++k)
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                     : "+d"(c0[k]), "+d"(c1[k]) : "d"(a), "d"(b));
    }
    for (int k = 0; k < 4; ++k) r += c0[k] + c1[k];
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

__global__ void empty_kernel(int* p) { if (p && threadIdx.x == 0 && blockIdx.x == 0) p[0] += 1; }

int main() {
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, 0));
  printf("device %s sms %d cc %d.%d smem/block optin %zu l2 %d clock(kHz) %d\n", prop.name, prop.multiProcessorCount,
         prop.major, prop.minor, prop.sharedMemPerBlockOptin, prop.l2CacheSize, 2070000);
  int sms = prop.multiProcessorCount;
  double* dout; float* fout; int* ip;
  CK(cudaMalloc(&dout, sizeof(double) * sms * 8 * 1024));
  CK(cudaMalloc(&fout, sizeof(float) * sms * 8 * 1024));
  CK(cudaMalloc(&ip, sizeof(int) * 16));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms;
  // DFMA throughput: many blocks x 8 chains
  for (int bpsm : {1, 4, 8}) {
    int iters = 4096;
    dfma_tp<8><<<sms * bpsm, 256>>>(dout, 16, 1.0000001, 1e-9);
    CK(cudaDeviceSynchronize());
    cudaEventRecord(e0);
    dfma_tp<8><<<sms * bpsm, 256>>>(dout, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    double flops = 2.0 * 8 * iters * 256.0 * sms * bpsm;
    printf("DFMA tp blocks/sm=%d: %.3f ms -> %.3f TFLOP/s\n", bpsm, ms, flops / ms / 1e9);
  }
  // DFMA latency: 1 warp, 1 chain
  {
    int iters = 1 << 16;
    dfma_tp<1><<<1, 32>>>(dout, 16, 1.0000001, 1e-9);
    CK(cudaDeviceSynchronize());
    cudaEventRecord(e0);
    dfma_tp<1><<<1, 32>>>(dout, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("DFMA latency (1 warp 1 chain): %.3f ns per fma (%.1f cycles at %d MHz nominal)\n", ms * 1e6 / iters,
           ms * 1e6 / iters * 2070000 / 1e6, 2070);
  }
  // DFMA one warp with 8 chains (per-SM issue of one warp)
  {
    int iters = 1 << 14;
    cudaEventRecord(e0);
    dfma_tp<8><<<1, 32>>>(dout, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("DFMA 1 warp 8 chains: %.3f ns per warp-fma\n", ms * 1e6 / iters / 8);
  }
  // DFMA 1 block of 256 threads x8 chains (one SM)
  {
    int iters = 1 << 12;
    cudaEventRecord(e0);
    dfma_tp<8><<<1, 256>>>(dout, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("DFMA 1 SM (256 thr x 8 chains): %.3f GFLOP/s per SM\n", 2.0 * 8 * iters * 256 / ms / 1e6);
  }
  // FFMA throughput
  {
    int iters = 4096;
    ffma_tp<8><<<sms * 4, 256>>>(fout, 16, 1.0000001f, 1e-9f);
    CK(cudaDeviceSynchronize());
    cudaEventRecord(e0);
    ffma_tp<8><<<sms * 4, 256>>>(fout, iters, 1.0000001f, 1e-9f);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("FFMA tp: %.3f TFLOP/s\n", 2.0 * 8 * iters * 256.0 * sms * 4 / ms / 1e9);
  }
  // DMMA throughput
  {
    int iters = 1024;
    dmma_tp<<<sms * 4, 256>>>(dout, 4);
    CK(cudaDeviceSynchronize());
    cudaEventRecord(e0);
    dmma_tp<<<sms * 4, 256>>>(dout, iters);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    double flops = 2.0 * 8 * 8 * 4 * 4.0 * iters * (256 / 32) * sms * 4;
    printf("DMMA m8n8k4 tp: %.3f TFLOP/s\n", flops / ms / 1e9);
  }
  // DFMA and DMMA warps side by side in every block: each half alone, then both
  for (int mode = 1; mode <= 3; ++mode) {
    const int iters = 2000, blocks = sms * 4;
    mixed<<<blocks, 256>>>(dout, 10, mode);
    CK(cudaDeviceSynchronize());
    cudaEventRecord(e0);
    mixed<<<blocks, 256>>>(dout, iters, mode);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    double fl_fma = (mode & 1) ? 4.0 * 32 * iters * 4 * 8 * 2 * blocks : 0.0;
    double fl_mma = (mode & 2) ? 4.0 * iters * 4 * 512.0 * blocks : 0.0;
    printf("mixed %s: %.3f ms  DFMA %.3f TF  DMMA %.3f TF  total %.3f TFLOP/s\n",
           mode == 1 ? "DFMA warps only" : mode == 2 ? "DMMA warps only" : "DFMA + DMMA warps", ms, fl_fma / ms / 1e9,
           fl_mma / ms / 1e9, (fl_fma + fl_mma) / ms / 1e9);
  }
  // launch overhead: 1000 back-to-back empty kernels
  {
    cudaStream_t s; cudaStreamCreate(&s);
    for (int i = 0; i < 10; ++i) empty_kernel<<<1, 32, 0, s>>>(ip);
    CK(cudaStreamSynchronize(s));
    cudaEventRecord(e0, s);
    for (int i = 0; i < 1000; ++i) empty_kernel<<<1, 32, 0, s>>>(ip);
    cudaEventRecord(e1, s);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("stream launch: %.3f us per empty kernel\n", ms * 1e3 / 1000);
    cudaGraph_t g; cudaGraphExec_t ge;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeGlobal));
    for (int i = 0; i < 100; ++i) empty_kernel<<<1, 32, 0, s>>>(ip);
    CK(cudaStreamEndCapture(s, &g));
    CK(cudaGraphInstantiate(&ge, g, 0));
    CK(cudaGraphLaunch(ge, s));
    CK(cudaStreamSynchronize(s));
    cudaEventRecord(e0, s);
    for (int i = 0; i < 10; ++i) CK(cudaGraphLaunch(ge, s));
    cudaEventRecord(e1, s);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("graph: %.3f us per empty kernel node\n", ms * 1e3 / 1000);
    // graph with 152-block kernels
    cudaGraph_t g2; cudaGraphExec_t ge2;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeGlobal));
    for (int i = 0; i < 100; ++i) empty_kernel<<<sms * 2, 256, 0, s>>>(nullptr);
    CK(cudaStreamEndCapture(s, &g2));
    CK(cudaGraphInstantiate(&ge2, g2, 0));
    CK(cudaGraphLaunch(ge2, s));
    CK(cudaStreamSynchronize(s));
    cudaEventRecord(e0, s);
    for (int i = 0; i < 10; ++i) CK(cudaGraphLaunch(ge2, s));
    cudaEventRecord(e1, s);
    CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms, e0, e1);
    printf("graph: %.3f us per empty 304x256 kernel node\n", ms * 1e3 / 1000);
  }
  CK(cudaDeviceSynchronize());
  printf("done\n");
  return 0;
}
