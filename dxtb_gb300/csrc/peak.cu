// FP64 throughput microbenchmarks: the roofline denominator for the
// engine's FP64-bound kernels (the machine's measured peaks cover HBM copy
// bandwidth and bf16 tensor throughput only), and the FP64 tensor-core
// (DMMA) rate, which decides whether FP64 panel updates would gain from
// running as warp-level MMA instead of DFMA.  Every thread (warp) runs 8
// independent DFMA (MMA) chains; the grid fills every SM with 8 blocks of
// 256 threads.  No counterpart in the reference.
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

// 8 independent m8n8k4 FP64 MMA chains per warp (512 flops per MMA)
__global__ void __launch_bounds__(256) k_dmma(double *out, int iters, double a, double b) {
  double c[8][2];
#pragma unroll
  for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = threadIdx.x * 1e-9 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
  if (s == 1.2345) out[0] = s;  // keeps the chains alive
}

// time one launch of kernel `f` (after a short warm-up) in milliseconds
template <typename F>
cudaError_t time_probe(F f, int iters, float *ms) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  f(iters / 8);  // warm-up
  cudaEventRecord(e0);
  f(iters);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  if (err == cudaSuccess) err = cudaGetLastError();
  cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return err;
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
  const int blocks = sms * 8, threads = 256, iters = 4096;
  float ms = 0.f;
  cudaError_t err = gbxtb::time_probe(
      [&](int it) { gbxtb::k_dfma<<<blocks, threads>>>(out, it, 0.9999999, 1e-7); }, iters, &ms);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return GBXTB_ERR_CUDA;
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *gflops = flops / (ms * 1e-3) / 1e9;
  return GBXTB_OK;
}

extern "C" GBXTB_API int gbxtb_fp64_mma_peak(double *gflops) {
  if (!gflops) return GBXTB_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GBXTB_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GBXTB_ERR_CUDA;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return GBXTB_ERR_CUDA;
  const int blocks = sms * 8, threads = 256, iters = 1024;
  float ms = 0.f;
  cudaError_t err =
      gbxtb::time_probe([&](int it) { gbxtb::k_dmma<<<blocks, threads>>>(out, it, 1e-3, 1e-3); }, iters, &ms);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return GBXTB_ERR_CUDA;
  // 8 MMAs of 8 x 8 x 4 multiply-adds per warp and iteration
  const double flops = 2.0 * 256.0 * 8.0 * (double)iters * blocks * (threads / 32);
  *gflops = flops / (ms * 1e-3) / 1e9;
  return GBXTB_OK;
}
