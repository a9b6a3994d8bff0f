// kf_fit_mixed.cu — mixed form (FP32 propagation and Jacobians, FP64 Kalman
// algebra): grid kernel and the default persistent kernel.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

cudaError_t launchFitMixed(const kfd::Params &P, unsigned grid, cudaStream_t s) {
  kfd::fitGrid<kfd::kFitBlock, KF_MIN_BLOCKS_MIXED, float><<<grid, kfd::kFitBlock, kfd::coldStateBytes<float>(), s>>>(P);
  return cudaGetLastError();
}

KF_PERSISTENT_LAUNCHER(launchPersistent_mixed_128_4, 128, 4, float)
