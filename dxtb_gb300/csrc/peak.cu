// FP64 FMA throughput microbenchmark: the roofline denominator for the
// engine's FP64-bound kernels (the machine's measured peaks cover HBM copy
// bandwidth and bf16 tensor throughput only).  Every thread runs 8
// independent DFMA chains; the grid fills every SM with 8 blocks of 256
// threads.  No counterpart in the reference.
#include "internal.cuh"

namespace gbxtb {
namespace {

__global__ void __launch_bounds__(256) k_dfma(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 1.2345) out[0] = s;  // keeps the chains alive
}

}  // namespace
}  // namespace gbxtb

extern "C" GBXTB_API int gbxtb_fp64_peak(double *gflops) {
  if (!gflops) return GBXTB_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GBXTB_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GBXTB_ERR_CUDA;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return GBXTB_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  gbxtb::k_dfma<<<blocks, threads>>>(out, iters / 8, 0.9999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  gbxtb::k_dfma<<<blocks, threads>>>(out, iters, 0.9999999, 1e-7);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return GBXTB_ERR_CUDA;
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *gflops = flops / (ms * 1e-3) / 1e9;
  return GBXTB_OK;
}
