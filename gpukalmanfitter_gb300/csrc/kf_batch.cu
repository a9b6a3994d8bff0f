// kf_batch.cu — the batched form: length-sorted work queue, persistent fit
// kernel, CUDA-graph plan and autotuner.
//
// The reference fits one track per GPU thread or block with one launch per
// stream (Run/GPU/Kernels.cu:6-94, Run/GPU/KalmanFitterGPUTest.cu:461-472); tracks
// of very different length share warps and the grid's tail idles.  Here the
// tracks are first ordered by expected work (sequence length, then |q/p|),
// longest first, by a counting sort over 2048 buckets; warps of a persistent
// grid then claim 32 consecutive queue positions at a time, so a warp holds
// tracks of similar length and the longest tracks start first.

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <new>

#include "kf_host.h"
#include "kf_kernels.cuh"

using namespace kfd;
using namespace kfh;

// persistent-kernel instantiations (kf_fit_*.cu, kf_tune_*.cu): launcher and
// shared-memory set-up
cudaError_t launchPersistent_fp64_128_4(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_fp64_128_4_prep();
cudaError_t launchPersistent_fp64_128_2(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_fp64_128_2_prep();
cudaError_t launchPersistent_fp64_128_3(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_fp64_128_3_prep();
cudaError_t launchPersistent_fp64_128_5(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_fp64_128_5_prep();
cudaError_t launchPersistent_fp64_64_4(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_fp64_64_4_prep();
cudaError_t launchPersistent_fp64_64_8(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_fp64_64_8_prep();
cudaError_t launchPersistent_fp64_256_1(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_fp64_256_1_prep();
cudaError_t launchPersistent_fp64_256_2(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_fp64_256_2_prep();
cudaError_t launchPersistent_mixed_128_4(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_mixed_128_4_prep();
cudaError_t launchPersistent_mixed_128_2(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_mixed_128_2_prep();
cudaError_t launchPersistent_mixed_128_3(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_mixed_128_3_prep();
cudaError_t launchPersistent_mixed_128_5(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_mixed_128_5_prep();
cudaError_t launchPersistent_mixed_64_4(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_mixed_64_4_prep();
cudaError_t launchPersistent_mixed_64_8(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_mixed_64_8_prep();
cudaError_t launchPersistent_mixed_256_1(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_mixed_256_1_prep();
cudaError_t launchPersistent_mixed_256_2(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_mixed_256_2_prep();
cudaError_t launchPersistent_fp64_mat(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_fp64_mat_prep();
cudaError_t launchPersistent_mixed_mat(const kfd::Params &, cudaStream_t);
cudaError_t launchPersistent_mixed_mat_prep();

namespace {

struct Variant {
  int precision, bs, minb;
  cudaError_t (*launch)(const Params &, cudaStream_t);
  cudaError_t (*prep)();
};
// (threads per CTA, CTAs per SM): register budgets 255 (128x2, 64x4, 256x1),
// 168 (128x3), 128 (128x4, 64x8, 256x2), 96 (128x5)
const Variant kVariants[] = {
    {KF_PRECISION_FP64, 128, 4, launchPersistent_fp64_128_4, launchPersistent_fp64_128_4_prep},
    {KF_PRECISION_FP64, 128, 2, launchPersistent_fp64_128_2, launchPersistent_fp64_128_2_prep},
    {KF_PRECISION_FP64, 128, 3, launchPersistent_fp64_128_3, launchPersistent_fp64_128_3_prep},
    {KF_PRECISION_FP64, 128, 5, launchPersistent_fp64_128_5, launchPersistent_fp64_128_5_prep},
    {KF_PRECISION_FP64, 64, 4, launchPersistent_fp64_64_4, launchPersistent_fp64_64_4_prep},
    {KF_PRECISION_FP64, 64, 8, launchPersistent_fp64_64_8, launchPersistent_fp64_64_8_prep},
    {KF_PRECISION_FP64, 256, 1, launchPersistent_fp64_256_1, launchPersistent_fp64_256_1_prep},
    {KF_PRECISION_FP64, 256, 2, launchPersistent_fp64_256_2, launchPersistent_fp64_256_2_prep},
    {KF_PRECISION_MIXED, 128, 4, launchPersistent_mixed_128_4, launchPersistent_mixed_128_4_prep},
    {KF_PRECISION_MIXED, 128, 2, launchPersistent_mixed_128_2, launchPersistent_mixed_128_2_prep},
    {KF_PRECISION_MIXED, 128, 3, launchPersistent_mixed_128_3, launchPersistent_mixed_128_3_prep},
    {KF_PRECISION_MIXED, 128, 5, launchPersistent_mixed_128_5, launchPersistent_mixed_128_5_prep},
    {KF_PRECISION_MIXED, 64, 4, launchPersistent_mixed_64_4, launchPersistent_mixed_64_4_prep},
    {KF_PRECISION_MIXED, 64, 8, launchPersistent_mixed_64_8, launchPersistent_mixed_64_8_prep},
    {KF_PRECISION_MIXED, 256, 1, launchPersistent_mixed_256_1, launchPersistent_mixed_256_1_prep},
    {KF_PRECISION_MIXED, 256, 2, launchPersistent_mixed_256_2, launchPersistent_mixed_256_2_prep},
};

// with material effects: the one instantiation with the material code
// (128 threads, 4 CTAs per SM), whatever the shape fields say
const Variant kMaterialVariants[] = {
    {KF_PRECISION_FP64, 128, 4, launchPersistent_fp64_mat, launchPersistent_fp64_mat_prep},
    {KF_PRECISION_MIXED, 128, 4, launchPersistent_mixed_mat, launchPersistent_mixed_mat_prep},
};

// the instantiation for a configuration (block size 0/128, min blocks 0 = 4)
const Variant *findVariant(const kf_config_t *cfg) {
  if (cfg->material_effects) {
    for (const Variant &v : kMaterialVariants)
      if (v.precision == cfg->precision) return &v;
    return nullptr;
  }
  const int bs = cfg->block_size ? cfg->block_size : 128;
  const int mb = cfg->min_blocks_per_sm ? cfg->min_blocks_per_sm : 4;
  for (const Variant &v : kVariants)
    if (v.precision == cfg->precision && v.bs == bs && v.minb == mb) return &v;
  return nullptr;
}

constexpr int kBuckets = kSortBuckets;

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct BatchLayout {
  size_t ws, perm, hist, offs, counter, total;
};
BatchLayout batchLayout(int64_t n, int32_t S, bool material) {
  BatchLayout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o = align256(o + bytes);
    return at;
  };
  L.ws = take(wsBytes(n, S, material));
  L.perm = take((size_t)n * sizeof(int32_t));
  L.hist = take(kBuckets * sizeof(int32_t));
  L.offs = take(kBuckets * sizeof(int32_t));
  L.counter = take(sizeof(int32_t));
  L.total = o;
  return L;
}

// Ascending key = descending expected work: sequence length first, then
// |q/p| on a log scale (steps per mm grow with curvature).
__device__ __forceinline__ int workKey(const Params &P, int64_t i) {
  int L = P.nplanes ? P.nplanes[i] : P.nSurf;
  L = min(max(L, 0), P.nSurf);
  const float qop = (float)fabs(P.start[4 * P.stride + i]);
  int qb = 0;
  if (qop > 0.f && qop < 3.0e38f) qb = (int)floorf((log2f(qop) + 7.f) * 2.f);
  qb = min(max(qb, 0), 15);
  return (64 - L) * 16 + (15 - qb);
}

__global__ void keyHistogram(const __grid_constant__ Params P, int32_t *hist) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P.n) atomicAdd(&hist[workKey(P, i)], 1);
}

// exclusive scan of kBuckets counts by one CTA of 1024 threads
__global__ void __launch_bounds__(1024) scanOffsets(const int32_t *hist, int32_t *offs) {
  __shared__ int32_t part[1024];
  const int t = threadIdx.x;
  const int a = hist[2 * t], b = hist[2 * t + 1];
  part[t] = a + b;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {
    const int v = (t >= d) ? part[t - d] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  const int before = part[t] - (a + b);
  offs[2 * t] = before;
  offs[2 * t + 1] = before + a;
}

__global__ void scatterPerm(const __grid_constant__ Params P, int32_t *offs, int32_t *perm) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P.n) perm[atomicAdd(&offs[workKey(P, i)], 1)] = (int32_t)i;
}

} // namespace

int32_t kfh::sortQueue(const Params &P, int32_t *hist, int32_t *offs, int32_t *perm,
                       cudaStream_t s) {
  if (P.n == 0) return KF_SUCCESS;
  cudaError_t e = cudaMemsetAsync(hist, 0, kBuckets * sizeof(int32_t), s);
  if (e != cudaSuccess) return cudaFail(e, "work-queue reset");
  const unsigned g = (unsigned)((P.n + 255) / 256);
  keyHistogram<<<g, 256, 0, s>>>(P, hist);
  scanOffsets<<<1, 1024, 0, s>>>(hist, offs);
  scatterPerm<<<g, 256, 0, s>>>(P, offs, perm);
  e = cudaGetLastError();
  return e == cudaSuccess ? KF_SUCCESS : cudaFail(e, "work-queue sort");
}

namespace {

int32_t enqueueBatched(const Params &P, const Variant *v, char *base, const BatchLayout &L,
                       cudaStream_t s) {
  if (P.n == 0) return KF_SUCCESS;
  HostRange range("work-queue sort + persistent fit");
  cudaError_t e = cudaMemsetAsync(base + L.counter, 0, sizeof(int32_t), s);
  if (e != cudaSuccess) return cudaFail(e, "batched queue reset");
  const int32_t rc = sortQueue(P, reinterpret_cast<int32_t *>(base + L.hist),
                               reinterpret_cast<int32_t *>(base + L.offs),
                               reinterpret_cast<int32_t *>(base + L.perm), s);
  if (rc) return rc;
  e = v->launch(P, s);
  if (e != cudaSuccess) return cudaFail(e, "persistent fit launch");
  return KF_SUCCESS;
}

int32_t prepare(const kf_inputs_t *in, kf_outputs_t *out, const kf_config_t *cfg,
                const kf_geometry_t *geo, const kf_field_t *field, void *workspace,
                size_t bytes, Params &P, const Variant *&v, BatchLayout &L) {
  int32_t rc = checkCommon(in, cfg, geo, field);
  if (rc) return rc;
  if (!out || !out->params || !out->cov || !out->chi2 || !out->status || !out->n_meas)
    return fail(KF_ERR_INVALID_ARGUMENT, "missing output array%s");
  if (in->n_tracks > 0 && (!in->meas || !in->start_params || !in->start_cov || !in->perigee))
    return fail(KF_ERR_INVALID_ARGUMENT, "missing input array%s");
  // the int32 queue counter runs up to n + 32 x (resident warps)
  if (in->n_tracks > 0x7f000000LL) return fail(KF_ERR_INVALID_ARGUMENT, "batch above 2^31 - 2^24 tracks%s");
  v = findVariant(cfg);
  if (!v) return fail(KF_ERR_UNSUPPORTED, "no persistent kernel for this block size / CTAs per SM%s");
  {
    const cudaError_t e = v->prep();
    if (e != cudaSuccess) return cudaFail(e, "persistent kernel shared-memory set-up");
  }
  L = batchLayout(in->n_tracks, in->n_surfaces, cfg->material_effects != 0);
  if (in->n_tracks > 0 && (!workspace || bytes < L.total))
    return fail(KF_ERR_WORKSPACE_TOO_SMALL, "workspace smaller than kf_batch_workspace_size()%s");
  char *base = static_cast<char *>(workspace);
  fillParams(P, in, out, cfg, geo, field, base + L.ws);
  P.perm = reinterpret_cast<const int32_t *>(base + L.perm);
  P.queueCounter = reinterpret_cast<int32_t *>(base + L.counter);
  return KF_SUCCESS;
}

} // namespace

struct kf_batch_plan {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" {

size_t kf_batch_workspace_size(const kf_config_t *cfg, int64_t n_tracks, int32_t n_surfaces) {
  (void)cfg;
  if (n_tracks <= 0 || n_surfaces <= 0) return 0;
  return batchLayout(n_tracks, n_surfaces, cfg && cfg->material_effects).total;
}

int32_t kf_fit_batch_sorted(const kf_inputs_t *in, kf_outputs_t *out, const kf_config_t *cfg,
                            const kf_geometry_t *geo, const kf_field_t *field, void *workspace,
                            size_t workspace_bytes, void *stream) {
  Params P;
  const Variant *v = nullptr;
  BatchLayout L;
  int32_t rc = prepare(in, out, cfg, geo, field, workspace, workspace_bytes, P, v, L);
  if (rc) return rc;
  return enqueueBatched(P, v, static_cast<char *>(workspace), L, static_cast<cudaStream_t>(stream));
}

int32_t kf_batch_plan_create(kf_batch_plan_t **plan, const kf_inputs_t *in, kf_outputs_t *out,
                             const kf_config_t *cfg, const kf_geometry_t *geo,
                             const kf_field_t *field, void *workspace, size_t workspace_bytes,
                             void *stream) {
  if (!plan) return fail(KF_ERR_INVALID_ARGUMENT, "null plan pointer%s");
  *plan = nullptr;
  if (!stream) return fail(KF_ERR_INVALID_ARGUMENT, "a plan needs a created stream (not the legacy default stream)%s");
  Params P;
  const Variant *v = nullptr;
  BatchLayout L;
  int32_t rc = prepare(in, out, cfg, geo, field, workspace, workspace_bytes, P, v, L);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cudaFail(e, "stream capture begin");
  rc = enqueueBatched(P, v, static_cast<char *>(workspace), L, s);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(s, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cudaFail(e, "stream capture end");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cudaFail(e, "graph instantiate");
  }
  kf_batch_plan *p = new (std::nothrow) kf_batch_plan;
  if (!p) {
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    return fail(KF_ERR_INVALID_ARGUMENT, "out of host memory%s");
  }
  p->graph = graph;
  p->exec = exec;
  *plan = p;
  return KF_SUCCESS;
}

int32_t kf_batch_plan_launch(kf_batch_plan_t *plan, void *stream) {
  HostRange range("kf_batch_plan_launch");
  if (!plan || !plan->exec) return fail(KF_ERR_INVALID_ARGUMENT, "null plan%s");
  cudaError_t e = cudaGraphLaunch(plan->exec, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cudaFail(e, "graph launch");
  return KF_SUCCESS;
}

void kf_batch_plan_destroy(kf_batch_plan_t *plan) {
  if (!plan) return;
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  if (plan->graph) cudaGraphDestroy(plan->graph);
  delete plan;
}

int32_t kf_autotune(const kf_inputs_t *in, kf_outputs_t *out, const kf_config_t *cfg,
                    const kf_geometry_t *geo, const kf_field_t *field, void *workspace,
                    size_t workspace_bytes, void *stream, kf_config_t *tuned, double *best_ms) {
  if (!in || !cfg || !tuned) return fail(KF_ERR_INVALID_ARGUMENT, "null argument%s");
  HostRange range("kf_autotune");
  // The first tracks (same stride) as the sample: at least several waves of
  // the resident grid, so that the queue's tail does not decide the timing.
  kf_inputs_t sample = *in;
  if (sample.n_tracks > 524288) sample.n_tracks = 524288;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return cudaFail(cudaGetLastError(), "event create");
  double best = 1e300;
  kf_config_t bestCfg = *cfg;
  int32_t rc = KF_SUCCESS;
  for (const Variant &v : kVariants) {
    if (v.precision != cfg->precision) continue;
    // with material effects the one material instantiation (128 x 4) runs
    if (cfg->material_effects && (v.bs != 128 || v.minb != 4)) continue;
    kf_config_t c = *cfg;
    c.kernel = KF_KERNEL_PERSISTENT;
    c.block_size = v.bs;
    c.min_blocks_per_sm = v.minb;
    rc = kf_fit_batch_sorted(&sample, out, &c, geo, field, workspace, workspace_bytes, stream);
    // best of three timed runs after one warm-up
    for (int r = 0; r < 3 && rc == KF_SUCCESS; ++r) {
      cudaEventRecord(e0, s);
      rc = kf_fit_batch_sorted(&sample, out, &c, geo, field, workspace, workspace_bytes, stream);
      cudaEventRecord(e1, s);
      if (rc) break;
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = cudaFail(cudaGetLastError(), "autotune timing");
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        bestCfg = c;
      }
    }
    if (rc) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  *tuned = bestCfg;
  if (best_ms) *best_ms = best;
  return KF_SUCCESS;
}

} // extern "C"
