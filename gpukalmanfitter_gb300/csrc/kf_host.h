// kf_host.h — host-side helpers shared by the C ABI translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "kf_device.cuh"

namespace kfh {

// A named range on a profiler's host timeline around one phase of a call
// (NVTX, header-only; without an attached tool a push or pop is a no-op
// check).  The reference marks its fit the same way (PUSH_RANGE / POP_RANGE,
// Utilities/Profiling.hpp:4-36, around Fitter/KalmanFitter.hpp:728-758).
struct HostRange {
  explicit HostRange(const char *name) { nvtxRangePushA(name); }
  ~HostRange() { nvtxRangePop(); }
  HostRange(const HostRange &) = delete;
  HostRange &operator=(const HostRange &) = delete;
};

char *errorBuffer(); // thread-local text behind kf_last_error_string()
int32_t fail(int32_t code, const char *fmt, const char *detail = "");
int32_t cudaFail(cudaError_t e, const char *where);

// bytes of the per-state smoother workspace of n tracks (with material: the
// covariances of the general smoother too)
size_t wsBytes(int64_t n, int32_t nSurf, bool material);
// argument checks shared by every fit entry point
int32_t checkCommon(const kf_inputs_t *in, const kf_config_t *cfg, const kf_geometry_t *geo,
                    const kf_field_t *field);
// work-queue order of P.n tracks (kf_batch.cu): perm[position] = track, longest
// and most curved first; hist and offs hold kSortBuckets ints each
constexpr int kSortBuckets = 2048;
int32_t sortQueue(const kfd::Params &P, int32_t *hist, int32_t *offs, int32_t *perm,
                  cudaStream_t s);
// kernel parameter block from the ABI structures
void fillParams(kfd::Params &P, const kf_inputs_t *in, const kf_outputs_t *out,
                const kf_config_t *cfg, const kf_geometry_t *geo, const kf_field_t *field,
                void *ws);

} // namespace kfh
