// kf_capi.cu — fit kernels and the C ABI declared in include/gb300kf.h.
//
// kf_fit_batch replaces the reference's per-track KalmanFitter::fit call
// (Fitter/KalmanFitter.hpp:716-768) and its launch by fitKernelThreadPerTrack
// (Run/GPU/Kernels.cu:6-45): one thread per track, structure-of-arrays inputs,
// no allocation, stream-ordered.

#include <cuda_runtime.h>

#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>

#include "kf_host.h"
#include "kf_kernels.cuh"

using namespace kfd;

// defined in kf_fit_fp64.cu / kf_fit_mixed.cu (one instantiation each, so the
// two compile in parallel)
cudaError_t launchFitFp64(const kfd::Params &P, unsigned grid, cudaStream_t s);
cudaError_t launchFitMixed(const kfd::Params &P, unsigned grid, cudaStream_t s);
cudaError_t launchFitFp64Mat(const kfd::Params &P, unsigned grid, cudaStream_t s);
cudaError_t launchFitMixedMat(const kfd::Params &P, unsigned grid, cudaStream_t s);

namespace {
thread_local char g_err[512] = "";
} // namespace

namespace kfh {

char *errorBuffer() { return g_err; }

int32_t fail(int32_t code, const char *fmt, const char *detail) {
  std::snprintf(g_err, sizeof(g_err), fmt, detail);
  return code;
}

int32_t cudaFail(cudaError_t e, const char *where) {
  std::snprintf(g_err, sizeof(g_err), "%s: %s", where, cudaGetErrorString(e));
  return KF_ERR_CUDA;
}

size_t wsBytes(int64_t n, int32_t nSurf, bool material) {
  // per state: predicted and filtered parameters and the Jacobian; with
  // material also the predicted and filtered covariance (general smoother)
  return (size_t)nSurf * (kStateStride + (material ? 42 : 0)) * (size_t)n * sizeof(double);
}

int32_t checkCommon(const kf_inputs_t *in, const kf_config_t *cfg, const kf_geometry_t *geo,
                    const kf_field_t *field) {
  if (!in || !cfg || !geo || !field) return fail(KF_ERR_INVALID_ARGUMENT, "null argument%s");
  if (in->n_tracks < 0 || in->stride < in->n_tracks)
    return fail(KF_ERR_INVALID_ARGUMENT, "bad n_tracks/stride%s");
  if (in->n_surfaces <= 0 || in->n_surfaces > KF_MAX_PLANES || geo->n_planes < in->n_surfaces)
    return fail(KF_ERR_INVALID_ARGUMENT, "bad n_surfaces (1..64, <= geometry planes)%s");
  if (!geo->center || !geo->rotation) return fail(KF_ERR_INVALID_ARGUMENT, "null geometry%s");
  if (field->kind != KF_FIELD_CONSTANT && field->kind != KF_FIELD_GRID3D &&
      field->kind != KF_FIELD_GRID_RZ)
    return fail(KF_ERR_INVALID_ARGUMENT, "unknown field kind%s");
  if (field->kind == KF_FIELD_GRID3D &&
      (!field->grid || field->nx < 2 || field->ny < 2 || field->nz < 2))
    return fail(KF_ERR_INVALID_ARGUMENT, "bad field grid%s");
  if (field->kind == KF_FIELD_GRID_RZ &&
      (!field->grid || field->nx < 2 || field->nz < 2 || !(field->max[0] > field->min[0]) ||
       !(field->max[2] > field->min[2])))
    return fail(KF_ERR_INVALID_ARGUMENT, "bad (r, z) field grid%s");
  if (cfg->precision != KF_PRECISION_FP64 && cfg->precision != KF_PRECISION_MIXED)
    return fail(KF_ERR_UNSUPPORTED, "unknown precision mode%s");
  if (cfg->max_steps < 0 || cfg->max_rk_trials < 0)
    return fail(KF_ERR_INVALID_ARGUMENT, "negative step limits%s");
  return KF_SUCCESS;
}

void fillParams(Params &P, const kf_inputs_t *in, const kf_outputs_t *out, const kf_config_t *cfg,
                const kf_geometry_t *geo, const kf_field_t *field, void *ws) {
  std::memset(&P, 0, sizeof(P));
  P.n = in->n_tracks;
  P.stride = in->stride;
  P.wsStride = in->n_tracks;
  P.nSurf = in->n_surfaces;
  P.maxSteps = cfg->max_steps;
  P.maxTrials = cfg->max_rk_trials;
  P.smoothing = cfg->smoothing;
  P.faithful = cfg->faithful_jacobian;
  P.tol = cfg->tolerance;
  P.cutoff = cfg->step_size_cutoff;
  P.mass = cfg->mass;
  P.overstep = cfg->overstep_limit;
  P.surfTol = cfg->on_surface_tol;
  P.outlierCut = cfg->outlier_chi2_cut;
  P.meas = in->meas;
  P.mask = in->hit_mask;
  P.nplanes = in->n_planes;
  P.start = in->start_params;
  P.scov = in->start_cov;
  P.perigee = in->perigee;
  P.oParams = out->params;
  P.oCov = out->cov;
  P.oChi2 = out->chi2;
  P.oSmoothed = out->smoothed;
  P.oStatus = out->status;
  P.oNMeas = out->n_meas;
  P.oNSteps = out->n_steps;
  P.oNTrials = out->n_trials;
  P.ws = static_cast<double *>(ws);
  FieldD &F = P.field;
  F.kind = field->kind;
  F.scale = field->scale;
  for (int a = 0; a < 3; ++a) {
    F.B[a] = field->value[a] * field->scale;
    F.mn[a] = field->min[a];
  }
  F.n[0] = field->nx;
  F.n[1] = field->ny;
  F.n[2] = field->nz;
  if (field->kind == KF_FIELD_GRID3D || field->kind == KF_FIELD_GRID_RZ) {
    for (int a = 0; a < 3; ++a) {
      const int na = (a == 0) ? field->nx : (a == 1) ? field->ny : field->nz;
      // the (r, z) grid has no y axis
      F.invw[a] = (field->kind == KF_FIELD_GRID_RZ && a == 1)
                      ? 0.
                      : (na - 1) / (field->max[a] - field->min[a]);
    }
  }
  F.grid = reinterpret_cast<const float4 *>(field->grid);
  for (int a = 0; a < 3; ++a) {
    F.Bf[a] = (float)F.B[a];
    F.Blo[a] = (float)(F.B[a] - (double)F.Bf[a]);
    F.mnf[a] = (float)F.mn[a];
    F.invwf[a] = (float)F.invw[a];
    F.wf[a] = (field->kind != KF_FIELD_CONSTANT && F.invw[a] != 0.) ? (float)(1. / F.invw[a]) : 0.f;
  }
  F.scalef = (float)F.scale;
  F.scalelo = (float)(F.scale - (double)F.scalef);
  P.tolLoF = (float)(P.tol * 0.99);
  for (int k = 0; k < in->n_surfaces; ++k) {
    PlaneD &pl = P.planes[k];
    for (int r = 0; r < 3; ++r) {
      pl.c[r] = geo->center[3 * k + r];
      pl.U[r] = geo->rotation[9 * k + 3 * r + 0];
      pl.V[r] = geo->rotation[9 * k + 3 * r + 1];
      pl.T[r] = geo->rotation[9 * k + 3 * r + 2];
    }
    {
      double m[6] = {0., 0., 0., 0., 0., 0.};
      if (geo->material)
        for (int e = 0; e < 6; ++e) m[e] = geo->material[6 * k + e];
      P.planeSlab[k] = kfm::slab(m);
    }
  }
  P.materialEffects = (geo->material && cfg->material_effects) ? (cfg->material_effects & 3) : 0;
  P.wsCov = cfg->material_effects
                ? static_cast<double *>(ws) + (size_t)in->n_surfaces * kStateStride * (size_t)P.wsStride
                : nullptr;
}

} // namespace kfh

using namespace kfh;

namespace {

int32_t launchFit(const Params &P, int precision, int blockSize, cudaStream_t s) {
  (void)blockSize;
  if (P.n == 0) return KF_SUCCESS;
  const unsigned grid = (unsigned)((P.n + kFitBlock - 1) / kFitBlock);
  const bool mat = P.materialEffects != 0;
  cudaError_t e = (precision == KF_PRECISION_MIXED)
                      ? (mat ? launchFitMixedMat(P, grid, s) : launchFitMixed(P, grid, s))
                      : (mat ? launchFitFp64Mat(P, grid, s) : launchFitFp64(P, grid, s));
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cudaFail(e, "fit kernel launch");
  return KF_SUCCESS;
}

} // namespace

extern "C" {

int32_t kf_version(void) { return KF_ABI_VERSION; }

const char *kf_last_error_string(void) { return g_err; }

void kf_config_default(kf_config_t *c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->precision = KF_PRECISION_FP64;
  c->max_steps = 1000;
  c->max_rk_trials = 10000;
  c->smoothing = 1;
  c->tolerance = 1e-4;
  c->step_size_cutoff = 0.;
  c->mass = 105.6583755e-3;
  c->overstep_limit = 0.01;
  c->on_surface_tol = 1e-4;
  c->outlier_chi2_cut = 0.;
  c->faithful_jacobian = 1;
  c->kernel = KF_KERNEL_AUTO;
  c->block_size = 0;
}

size_t kf_workspace_size(const kf_config_t *cfg, int64_t n_tracks, int32_t n_surfaces) {
  if (n_tracks <= 0 || n_surfaces <= 0) return 0;
  return wsBytes(n_tracks, n_surfaces, cfg && cfg->material_effects);
}

int32_t kf_fit_batch(const kf_inputs_t *in, kf_outputs_t *out, const kf_config_t *cfg,
                     const kf_geometry_t *geo, const kf_field_t *field, void *workspace,
                     size_t workspace_bytes, void *stream) {
  HostRange range("kf_fit_batch");
  int32_t rc = checkCommon(in, cfg, geo, field);
  if (rc) return rc;
  if (!out || !out->params || !out->cov || !out->chi2 || !out->status || !out->n_meas)
    return fail(KF_ERR_INVALID_ARGUMENT, "missing output array%s");
  if (in->n_tracks > 0 && (!in->meas || !in->start_params || !in->start_cov || !in->perigee))
    return fail(KF_ERR_INVALID_ARGUMENT, "missing input array%s");
  if (workspace_bytes < wsBytes(in->n_tracks, in->n_surfaces, cfg->material_effects != 0) ||
      (!workspace && in->n_tracks > 0))
    return fail(KF_ERR_WORKSPACE_TOO_SMALL, "workspace smaller than kf_workspace_size()%s");
  Params P;
  fillParams(P, in, out, cfg, geo, field, workspace);
  return launchFit(P, cfg->precision, cfg->block_size, static_cast<cudaStream_t>(stream));
}

// ---- host-buffer convenience ----------------------------------------------
namespace {
struct Staging {
  size_t meas, mask, nplanes, start, scov, perigee;
  size_t params, cov, chi2, status, nmeas, nsteps, ntrials, smoothed, ws, total;
};
size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
Staging stagingLayout(int64_t n, int32_t S, bool withSmoothed, const kf_config_t *cfg) {
  Staging L{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o = align256(o + bytes);
    return at;
  };
  L.meas = take((size_t)S * 5 * n * 8);
  L.mask = take((size_t)n * 8);
  L.nplanes = take((size_t)n * 4);
  L.start = take((size_t)6 * n * 8);
  L.scov = take((size_t)21 * n * 8);
  L.perigee = take((size_t)3 * n * 8);
  L.params = take((size_t)6 * n * 8);
  L.cov = take((size_t)21 * n * 8);
  L.chi2 = take((size_t)n * 8);
  L.status = take((size_t)n * 4);
  L.nmeas = take((size_t)n * 4);
  L.nsteps = take((size_t)n * 4);
  L.ntrials = take((size_t)n * 4);
  L.smoothed = withSmoothed ? take((size_t)S * 27 * n * 8) : 0;
  // room for either form's workspace (the batched form adds its queue)
  const bool mat = cfg && cfg->material_effects;
  L.ws = take(std::max(wsBytes(n, S, mat), kf_batch_workspace_size(cfg, n, S)));
  L.total = o;
  return L;
}

// copy `rows` rows of `n` elements from a host SoA with stride `hs` into a
// compact device SoA (or back)
cudaError_t copyRows(void *dst, size_t dpitchElems, const void *src, size_t spitchElems,
                     size_t elem, size_t n, size_t rows, cudaMemcpyKind kind, cudaStream_t s) {
  if (!rows || !n) return cudaSuccess;
  return cudaMemcpy2DAsync(dst, dpitchElems * elem, src, spitchElems * elem, n * elem, rows, kind, s);
}

constexpr int64_t kHostChunkMin = 131072; // tracks per chunk of a pipelined host call

// a second stream per device for the chunk pipeline, created once
cudaError_t auxStream(cudaStream_t *out) {
  static std::mutex mu;
  static cudaStream_t streams[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(mu);
  if (!streams[dev]) {
    e = cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      streams[dev] = nullptr;
      return e;
    }
  }
  *out = streams[dev];
  return cudaSuccess;
}

// tracks [c0, c0 + cn) of a host batch: copies in, fit, copies out, on stream
// s, with staging for cn tracks at d (no synchronisation)
int32_t hostChunk(const kf_inputs_t *hin, kf_outputs_t *hout, const kf_config_t *cfg,
                  const kf_geometry_t *geo, const kf_field_t *field, char *d, int64_t c0,
                  int64_t cn, cudaStream_t s) {
  const int32_t S = hin->n_surfaces;
  const bool sm = hout->smoothed != nullptr;
  const Staging L = stagingLayout(cn, S, sm, cfg);
  const size_t hs = (size_t)hin->stride;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  nvtxRangePushA("host-to-device copies");
  chk(copyRows(d + L.meas, cn, hin->meas + c0, hs, 8, cn, (size_t)S * 5, cudaMemcpyHostToDevice, s));
  if (hin->hit_mask)
    chk(cudaMemcpyAsync(d + L.mask, hin->hit_mask + c0, cn * 8, cudaMemcpyHostToDevice, s));
  if (hin->n_planes)
    chk(cudaMemcpyAsync(d + L.nplanes, hin->n_planes + c0, cn * 4, cudaMemcpyHostToDevice, s));
  chk(copyRows(d + L.start, cn, hin->start_params + c0, hs, 8, cn, 6, cudaMemcpyHostToDevice, s));
  chk(copyRows(d + L.scov, cn, hin->start_cov + c0, hs, 8, cn, 21, cudaMemcpyHostToDevice, s));
  chk(copyRows(d + L.perigee, cn, hin->perigee + c0, hs, 8, cn, 3, cudaMemcpyHostToDevice, s));
  nvtxRangePop();
  if (e != cudaSuccess) return cudaFail(e, "host-to-device copy");
  kf_inputs_t din = *hin;
  din.n_tracks = cn;
  din.stride = cn;
  din.meas = reinterpret_cast<const double *>(d + L.meas);
  din.hit_mask = hin->hit_mask ? reinterpret_cast<const uint64_t *>(d + L.mask) : nullptr;
  din.n_planes = hin->n_planes ? reinterpret_cast<const int32_t *>(d + L.nplanes) : nullptr;
  din.start_params = reinterpret_cast<const double *>(d + L.start);
  din.start_cov = reinterpret_cast<const double *>(d + L.scov);
  din.perigee = reinterpret_cast<const double *>(d + L.perigee);
  kf_outputs_t dout;
  dout.params = reinterpret_cast<double *>(d + L.params);
  dout.cov = reinterpret_cast<double *>(d + L.cov);
  dout.chi2 = reinterpret_cast<double *>(d + L.chi2);
  dout.status = reinterpret_cast<int32_t *>(d + L.status);
  dout.n_meas = reinterpret_cast<int32_t *>(d + L.nmeas);
  dout.n_steps = reinterpret_cast<int32_t *>(d + L.nsteps);
  dout.n_trials = reinterpret_cast<int32_t *>(d + L.ntrials);
  dout.smoothed = sm ? reinterpret_cast<double *>(d + L.smoothed) : nullptr;
  const size_t wsb = std::max(wsBytes(cn, S, cfg->material_effects != 0), kf_batch_workspace_size(cfg, cn, S));
  const int32_t rc = (cfg->kernel == KF_KERNEL_PERSISTENT)
                         ? kf_fit_batch_sorted(&din, &dout, cfg, geo, field, d + L.ws, wsb, s)
                         : kf_fit_batch(&din, &dout, cfg, geo, field, d + L.ws, wsb, s);
  if (rc) return rc;
  HostRange copiesOut("device-to-host copies");
  const size_t os = hs; // host outputs share the input stride
  chk(copyRows(hout->params + c0, os, dout.params, cn, 8, cn, 6, cudaMemcpyDeviceToHost, s));
  chk(copyRows(hout->cov + c0, os, dout.cov, cn, 8, cn, 21, cudaMemcpyDeviceToHost, s));
  chk(cudaMemcpyAsync(hout->chi2 + c0, dout.chi2, cn * 8, cudaMemcpyDeviceToHost, s));
  chk(cudaMemcpyAsync(hout->status + c0, dout.status, cn * 4, cudaMemcpyDeviceToHost, s));
  chk(cudaMemcpyAsync(hout->n_meas + c0, dout.n_meas, cn * 4, cudaMemcpyDeviceToHost, s));
  if (hout->n_steps)
    chk(cudaMemcpyAsync(hout->n_steps + c0, dout.n_steps, cn * 4, cudaMemcpyDeviceToHost, s));
  if (hout->n_trials)
    chk(cudaMemcpyAsync(hout->n_trials + c0, dout.n_trials, cn * 4, cudaMemcpyDeviceToHost, s));
  if (sm)
    chk(copyRows(hout->smoothed + c0, os, dout.smoothed, cn, 8, cn, (size_t)S * 27,
                 cudaMemcpyDeviceToHost, s));
  if (e != cudaSuccess) return cudaFail(e, "device-to-host copy");
  return KF_SUCCESS;
}
} // namespace

int32_t kf_material_interaction(const double mat[6], int32_t flags, const double normal[3],
                                const double dir[3], double p, double q, double mass,
                                double out[5]) {
  if (!mat || !normal || !dir || !out) return fail(KF_ERR_INVALID_ARGUMENT, "null argument%s");
  kfm::Effects e;
  if (!kfm::interact(mat, flags, normal, dir, p, q, mass, e)) return 1;
  out[0] = e.p;
  out[1] = e.varPhi;
  out[2] = e.varTheta;
  out[3] = e.varQop;
  out[4] = e.eloss;
  return KF_SUCCESS;
}

size_t kf_host_staging_size(const kf_config_t *cfg, int64_t n_tracks, int32_t n_surfaces,
                            int32_t with_smoothed) {
  if (n_tracks <= 0 || n_surfaces <= 0) return 0;
  return stagingLayout(n_tracks, n_surfaces, with_smoothed != 0, cfg).total;
}

int32_t kf_fit_batch_host(const kf_inputs_t *hin, kf_outputs_t *hout, const kf_config_t *cfg,
                          const kf_geometry_t *geo, const kf_field_t *field, void *dev,
                          size_t bytes, void *stream) {
  HostRange range("kf_fit_batch_host");
  int32_t rc = checkCommon(hin, cfg, geo, field);
  if (rc) return rc;
  if (!hout || !hout->params || !hout->cov || !hout->chi2 || !hout->status || !hout->n_meas)
    return fail(KF_ERR_INVALID_ARGUMENT, "missing output array%s");
  const int64_t n = hin->n_tracks;
  if (n == 0) return KF_SUCCESS;
  const int32_t S = hin->n_surfaces;
  const bool sm = hout->smoothed != nullptr;
  const Staging L = stagingLayout(n, S, sm, cfg);
  if (!dev || bytes < L.total)
    return fail(KF_ERR_WORKSPACE_TOO_SMALL, "staging smaller than kf_host_staging_size()%s");
  char *d = static_cast<char *>(dev);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Large batches run as K chunks alternating between the caller's stream and
  // a second stream of this device, so that one chunk's copies overlap
  // another chunk's fit; two staging slots of chunk size fit in the staging
  // area sized for the whole batch.
  int K = n >= 4 * kHostChunkMin ? 4 : (n >= 2 * kHostChunkMin ? 2 : 1);
  const int64_t chunk = (n + K - 1) / K;
  const size_t slot = stagingLayout(chunk, S, sm, cfg).total;
  cudaStream_t aux = nullptr;
  if (K > 1 && (2 * slot > bytes || auxStream(&aux) != cudaSuccess)) K = 1;
  if (K == 1) {
    rc = hostChunk(hin, hout, cfg, geo, field, d, 0, n, s);
    if (rc) return rc;
  } else {
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&ev0, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev1, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev0, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(aux, ev0, 0);
    if (e != cudaSuccess) return cudaFail(e, "chunk pipeline set-up");
    for (int k = 0; k < K && rc == KF_SUCCESS; ++k) {
      const int64_t c0 = k * chunk, cn = std::min(chunk, n - c0);
      if (cn <= 0) break;
      rc = hostChunk(hin, hout, cfg, geo, field, d + (k % 2) * slot, c0, cn, (k % 2) ? aux : s);
    }
    // the caller's stream continues after both streams' work
    e = cudaEventRecord(ev1, aux);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev1, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    if (rc) return rc;
    if (e != cudaSuccess) return cudaFail(e, "chunk pipeline");
    return KF_SUCCESS;
  }
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cudaFail(e, "stream synchronize");
  return KF_SUCCESS;
}

} // extern "C"
