// kf_tune_fp64_64x8.cu — persistent kernel, fp64 form, 64 threads per CTA and at least 8 CTAs
// per SM (register budget 65536 / (64 x 8)): an autotuner candidate.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

KF_PERSISTENT_LAUNCHER(launchPersistent_fp64_64_8, 64, 8, double)
