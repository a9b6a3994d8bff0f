// kf_fit_fp64.cu — plain form (FP64 throughout): grid kernel and the default
// persistent kernel.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

cudaError_t launchFitFp64(const kfd::Params &P, unsigned grid, cudaStream_t s) {
  kfd::fitGrid<kfd::kFitBlock, KF_MIN_BLOCKS_FP64, double><<<grid, kfd::kFitBlock, kfd::coldStateBytes<double>(), s>>>(P);
  return cudaGetLastError();
}

KF_PERSISTENT_LAUNCHER(launchPersistent_fp64_128_4, 128, 4, double)
