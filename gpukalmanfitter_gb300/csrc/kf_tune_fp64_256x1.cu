// kf_tune_fp64_256x1.cu — persistent kernel, fp64 form, 256 threads per CTA and at least 1 CTAs
// per SM (register budget 65536 / (256 x 1)): an autotuner candidate.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

KF_PERSISTENT_LAUNCHER(launchPersistent_fp64_256_1, 256, 1, double)
