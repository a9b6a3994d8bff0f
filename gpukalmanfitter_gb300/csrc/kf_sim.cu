// kf_sim.cu — the synthetic telescope workloads generated on the GPU
// (kf_simulate_tracks, gb300kf_synth.h): one thread per track running the
// host generator's per-track code (kf_synth_track.h), writing the fit's
// input arrays straight into device memory.
#include <cuda_runtime.h>

#include "kf_host.h"
#include "kf_synth_track.h"

namespace {

struct SimParams {
  kf_synth_config_t cfg;
  double tcenter[KF_MAX_PLANES * 3];
  double trot[KF_MAX_PLANES * 9];
  kfs::GridView grid;
  int useMap;
  double bz;
  int64_t n;
  kfs::TrackOut out;
};

constexpr int kSimThreads = 128;

__global__ void __launch_bounds__(kSimThreads) simulateKernel(const __grid_constant__ SimParams P) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += stride)
    kfs::simulateTrack(P.cfg, P.tcenter, P.trot, P.useMap ? &P.grid : nullptr, P.bz, i, P.n,
                       P.out);
}

} // namespace

extern "C" int32_t kf_simulate_tracks(const kf_synth_config_t *cfg, const double *truth_center,
                                      const double *truth_rotation, const kf_field_t *field,
                                      double *meas, uint64_t *hit_mask, int32_t *n_planes,
                                      double *start_params, double *start_cov, double *perigee,
                                      double *truth, void *stream) {
  if (!cfg) return kfh::fail(KF_ERR_INVALID_ARGUMENT, "kf_simulate_tracks: %s", "no config");
  if (cfg->n_tracks == 0) return KF_SUCCESS; // nothing to write (arrays may be NULL)
  if (!truth_center || !truth_rotation || !meas || !start_params || !start_cov || !perigee)
    return kfh::fail(KF_ERR_INVALID_ARGUMENT, "kf_simulate_tracks: %s", "missing array");
  const int S = cfg->n_planes;
  if (cfg->n_tracks < 0 || S <= 0 || S > KF_MAX_PLANES || cfg->min_len < 1 ||
      cfg->max_len > S || cfg->min_len > cfg->max_len)
    return kfh::fail(KF_ERR_INVALID_ARGUMENT, "kf_simulate_tracks: %s",
                     "bad track count, plane count or length range");
  const bool useMap = field && (field->kind == KF_FIELD_GRID3D || field->kind == KF_FIELD_GRID_RZ);
  const bool withMaterial = cfg->material[0] > 0. && cfg->material[3] > 0.;
  if (withMaterial && useMap)
    return kfh::fail(KF_ERR_UNSUPPORTED, "kf_simulate_tracks: %s",
                     "material truth needs the uniform field");
  if (useMap && (!field->grid || ((uintptr_t)field->grid & 15) || field->nx < 2 ||
                 field->ny < 2 || field->nz < 2))
    return kfh::fail(KF_ERR_INVALID_ARGUMENT, "kf_simulate_tracks: %s", "bad field grid");
  SimParams P;
  P.cfg = *cfg;
  for (int k = 0; k < 3 * S; ++k) P.tcenter[k] = truth_center[k];
  for (int k = 0; k < 9 * S; ++k) P.trot[k] = truth_rotation[k];
  P.useMap = useMap;
  if (useMap) P.grid = kfs::gridView(*field);
  P.bz = cfg->bz_tesla * kfs::kTesla * ((field && !useMap) ? field->scale : 1.0);
  P.n = cfg->n_tracks;
  P.out = kfs::TrackOut{meas, hit_mask, n_planes, start_params, start_cov, perigee, truth};
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return kfh::cudaFail(e, "kf_simulate_tracks");
  const int64_t want = (P.n + kSimThreads - 1) / kSimThreads;
  const int blocks = (int)std::min<int64_t>(want, (int64_t)sms * 16);
  simulateKernel<<<blocks, kSimThreads, 0, (cudaStream_t)stream>>>(P);
  e = cudaGetLastError();
  if (e != cudaSuccess) return kfh::cudaFail(e, "kf_simulate_tracks launch");
  return KF_SUCCESS;
}
