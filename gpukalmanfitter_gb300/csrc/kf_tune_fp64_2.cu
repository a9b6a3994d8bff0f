// kf_tune_fp64_2.cu — persistent kernel, fp64 form, 128 threads per CTA and
// at least 2 CTAs per SM (register budget 65536 / (128 x 2)): an autotuner
// candidate.
#include <cuda_runtime.h>

#include "kf_kernels.cuh"

KF_PERSISTENT_LAUNCHER(launchPersistent_fp64_128_2, 128, 2, double)
