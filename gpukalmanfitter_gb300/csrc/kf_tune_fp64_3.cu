// kf_tune_fp64_3.cu — persistent kernel, fp64 form, 128 threads per CTA and
// at least 3 CTAs per SM (register budget 65536 / (128 x 3)): an autotuner
// candidate.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

KF_PERSISTENT_LAUNCHER(launchPersistent_fp64_128_3, 128, 3, double)
