// kf_tune_mixed_64x8.cu — persistent kernel, mixed form, 64 threads per CTA and at least 8 CTAs
// per SM (register budget 65536 / (64 x 8)): an autotuner candidate.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

KF_PERSISTENT_LAUNCHER(launchPersistent_mixed_64_8, 64, 8, float)
