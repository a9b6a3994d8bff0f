// kf_fit_mixed_mat.cu — mixed form with surface material effects compiled in:
// grid kernel and the persistent kernel the batched form runs with material.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

cudaError_t launchFitMixedMat(const kfd::Params &P, unsigned grid, cudaStream_t s) {
  kfd::fitGrid<kfd::kFitBlock, KF_MIN_BLOCKS_MIXED, float, kfd::MaterialHook>
      <<<grid, kfd::kFitBlock, kfd::coldStateBytes<float>(), s>>>(P);
  return cudaGetLastError();
}

KF_PERSISTENT_LAUNCHER_H(launchPersistent_mixed_mat, 128, 4, float, kfd::MaterialHook)
