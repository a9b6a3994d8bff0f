// kf_tune_mixed_64x4.cu — persistent kernel, mixed form, 64 threads per CTA and at least 4 CTAs
// per SM (register budget 65536 / (64 x 4)): an autotuner candidate.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

KF_PERSISTENT_LAUNCHER(launchPersistent_mixed_64_4, 64, 4, float)
