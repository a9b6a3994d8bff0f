// kf_fit_fp64.cu — instantiation of the fit kernel for the plain form (FP64 throughout).
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

cudaError_t launchFitFp64(const kfd::Params &P, unsigned grid, cudaStream_t s) {
  kfd::fitKernel<kfd::kFitBlock, double><<<grid, kfd::kFitBlock, 0, s>>>(P);
  return cudaGetLastError();
}
