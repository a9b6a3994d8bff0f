// kf_tune_mixed_256x2.cu — persistent kernel, mixed form, 256 threads per CTA and at least 2 CTAs
// per SM (register budget 65536 / (256 x 2)): an autotuner candidate.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

KF_PERSISTENT_LAUNCHER(launchPersistent_mixed_256_2, 256, 2, float)
