// kf_fit_mixed.cu — instantiation of the fit kernel for the mixed form (FP32 propagation and Jacobians, FP64 Kalman algebra).
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

cudaError_t launchFitMixed(const kfd::Params &P, unsigned grid, cudaStream_t s) {
  kfd::fitKernel<kfd::kFitBlock, float><<<grid, kfd::kFitBlock, 0, s>>>(P);
  return cudaGetLastError();
}
