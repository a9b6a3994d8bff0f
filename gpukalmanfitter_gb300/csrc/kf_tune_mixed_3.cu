// kf_tune_mixed_3.cu — persistent kernel, mixed form, 128 threads per CTA and
// at least 3 CTAs per SM (register budget 65536 / (128 x 3)): an autotuner
// candidate.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

KF_PERSISTENT_LAUNCHER(launchPersistent_mixed_128_3, 128, 3, float)
