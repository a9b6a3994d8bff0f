// kf_kernels.cuh — fit kernels over the per-track state machine.
//
// fitGrid:       one thread per track, grid over the batch (kf_fit_batch).
// fitPersistent: the batched form.  A grid sized to the resident capacity of
//                the device; every warp claims 32 consecutive positions of a
//                work queue (tracks sorted longest first) with one atomic,
//                fits them, and claims again until the queue is empty.
//
// In both, lanes step independently and park at heavy actor work (filter
// update, smoothing, final transport); when every lane of the warp is parked
// or done, the parked lanes run their events together, so the FP64-heavy
// Kalman algebra executes without divergence.
#pragma once

#include "kf_device.cuh"

namespace kfd {

constexpr int kFitBlock = kLaneSlots; // threads per CTA of every fit kernel
#ifndef KF_MIN_BLOCKS_FP64
#define KF_MIN_BLOCKS_FP64 4
#endif
#ifndef KF_MIN_BLOCKS_MIXED
#define KF_MIN_BLOCKS_MIXED 4
#endif
template <typename R> struct MinBlocks {
  static constexpr int value = sizeof(R) == sizeof(double) ? KF_MIN_BLOCKS_FP64 : KF_MIN_BLOCKS_MIXED;
};

// Fit the tracks i (inputs/outputs) with workspace columns w of one warp;
// i < 0 marks an idle lane.  All 32 lanes must call it together.
template <typename R, typename H>
__device__ __forceinline__ void fitWarp(const Params &P, const PlaneD *sp, int64_t i, int64_t w) {
  Lane<R, H> L;
  initLane(L, P, sp, i, w);
  for (;;) {
    if (!L.parked && L.pc != PC_DONE) advance(L, P, sp);
    const bool waiting = L.parked || L.pc == PC_DONE;
    if (__all_sync(0xffffffffu, waiting)) {
      if (L.parked) runEvent(L, P, sp);
      if (__all_sync(0xffffffffu, L.pc == PC_DONE)) break;
    }
  }
  if (i >= 0 && i < P.n) {
    P.oStatus[i] = L.status;
    P.oChi2[i] = L.chi2;
    P.oNMeas[i] = L.measStates;
    if (P.oNSteps) P.oNSteps[i] = L.rkSteps;
    if (P.oNTrials) P.oNTrials[i] = L.rkTrials;
    if (L.status != KF_TRACK_OK && !L.finished) {
      for (int e = 0; e < 6; ++e) P.oParams[(size_t)e * P.stride + i] = 0.;
      for (int e = 0; e < 21; ++e) P.oCov[(size_t)e * P.stride + i] = 0.;
    }
  }
}

template <int BS, int MINB, typename R, typename H = NoHook>
__global__ void __launch_bounds__(BS, MINB) fitGrid(const __grid_constant__ Params P) {
  __shared__ PlaneD sp[KF_MAX_PLANES];
  for (int k = threadIdx.x; k < P.nSurf; k += BS) sp[k] = P.planes[k];
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * BS + threadIdx.x;
  fitWarp<R, H>(P, sp, i, i);
}

template <int BS, int MINB, typename R, typename H = NoHook>
__global__ void __launch_bounds__(BS, MINB) fitPersistent(const __grid_constant__ Params P) {
  __shared__ PlaneD sp[KF_MAX_PLANES];
  for (int k = threadIdx.x; k < P.nSurf; k += BS) sp[k] = P.planes[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(P.queueCounter, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if ((int64_t)base >= P.n) break;
    const int64_t q = (int64_t)base + lane;
    const int64_t i = (q < P.n) ? (int64_t)P.perm[q] : -1;
    fitWarp<R, H>(P, sp, i, q < P.n ? q : 0);
  }
}

} // namespace kfd

// Launcher of one instantiation of the persistent kernel: as many CTAs as the
// device holds at once (occupancy query), never more than the batch needs.
// NAME##_prep lifts the CTA's dynamic shared-memory limit to the cold state's
// size (needed above 48 KB); callers run it before any launch or capture.
#define KF_PERSISTENT_LAUNCHER(NAME, BS, MINB, R) KF_PERSISTENT_LAUNCHER_H(NAME, BS, MINB, R, kfd::NoHook)
#define KF_PERSISTENT_LAUNCHER_H(NAME, BS, MINB, R, H)                                         \
  cudaError_t NAME##_prep() {                                                                \
    return cudaFuncSetAttribute(kfd::fitPersistent<BS, MINB, R, H>,                          \
                                cudaFuncAttributeMaxDynamicSharedMemorySize,                 \
                                (int)kfd::coldStateBytes<R>(BS));                            \
  }                                                                                          \
  cudaError_t NAME(const kfd::Params &P, cudaStream_t s) {                                   \
    int dev = 0, sms = 0, per = 0;                                                           \
    cudaError_t e = cudaGetDevice(&dev);                                                     \
    if (e != cudaSuccess) return e;                                                          \
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);                   \
    if (e != cudaSuccess) return e;                                                          \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kfd::fitPersistent<BS, MINB, R, H>, \
                                                      BS, kfd::coldStateBytes<R>(BS));       \
    if (e != cudaSuccess) return e;                                                          \
    int64_t blocks = (int64_t)sms * (per > 0 ? per : 1);                                     \
    const int64_t need = (P.n + BS - 1) / BS;                                                \
    if (blocks > need) blocks = need;                                                        \
    if (blocks < 1) blocks = 1;                                                              \
    kfd::fitPersistent<BS, MINB, R, H><<<(unsigned)blocks, BS, kfd::coldStateBytes<R>(BS), s>>>(P); \
    return cudaGetLastError();                                                               \
  }
