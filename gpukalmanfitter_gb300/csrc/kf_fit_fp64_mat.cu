// kf_fit_fp64_mat.cu — plain form with surface material effects compiled in:
// grid kernel and the persistent kernel the batched form runs with material.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

cudaError_t launchFitFp64Mat(const kfd::Params &P, unsigned grid, cudaStream_t s) {
  kfd::fitGrid<kfd::kFitBlock, KF_MIN_BLOCKS_FP64, double, kfd::MaterialHook>
      <<<grid, kfd::kFitBlock, kfd::coldStateBytes<double>(), s>>>(P);
  return cudaGetLastError();
}

KF_PERSISTENT_LAUNCHER_H(launchPersistent_fp64_mat, 128, 4, double, kfd::MaterialHook)
