// kf_diag.cu — FP64 FMA throughput probe used as the roofline denominator.
#include <cuda_runtime.h>

#include "../../include/gb300kf.h"
#include "../../include/gb300kf_diag.h"

namespace {

__device__ double g_sink[256];

__global__ void __launch_bounds__(256) fmaChains(int iters, double seed) {
  double a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4,
         a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const double m = 0.999999999, c = 1e-9;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c);
    a1 = fma(a1, m, c);
    a2 = fma(a2, m, c);
    a3 = fma(a3, m, c);
    a4 = fma(a4, m, c);
    a5 = fma(a5, m, c);
    a6 = fma(a6, m, c);
    a7 = fma(a7, m, c);
  }
  const double r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == 12345.678) g_sink[threadIdx.x] = r; // keeps the chains live
}

} // namespace

extern "C" int32_t kf_diag_fp64_fma_rate(int32_t iters, double *gflops_out, void *stream) {
  if (!gflops_out || iters <= 0) return KF_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return KF_ERR_NO_DEVICE;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fmaChains<<<blocks, threads, 0, s>>>(iters / 10, 1.0); // warm-up
  cudaEventRecord(e0, s);
  fmaChains<<<blocks, threads, 0, s>>>(iters, 1.0);
  cudaEventRecord(e1, s);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess || cudaGetLastError() != cudaSuccess) return KF_ERR_CUDA;
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *gflops_out = flops / (ms * 1e-3) / 1e9;
  return KF_SUCCESS;
}
