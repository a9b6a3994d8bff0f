// kf_kernels.cuh — the fit kernel over the per-track state machine.
#pragma once

#include "kf_device.cuh"

namespace kfd {

constexpr int kFitBlock = 128; // threads per CTA

// Warp-synchronous driver: lanes step independently and park at heavy actor
// work (filter update, smoothing, final transport); when every lane of the
// warp is parked or done the parked lanes run their events together, so the
// FP64-heavy Kalman algebra executes without divergence.
// R = double: plain FP64 form; R = float: mixed form.
template <int BS, typename R>
__global__ void __launch_bounds__(BS) fitKernel(const __grid_constant__ Params P) {
  __shared__ PlaneD sp[KF_MAX_PLANES];
  for (int k = threadIdx.x; k < P.nSurf; k += BS) sp[k] = P.planes[k];
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * BS + threadIdx.x;
  Lane<R> L;
  initLane(L, P, sp, i);
  for (;;) {
    if (!L.parked && L.pc != PC_DONE) advance(L, P, sp);
    const bool waiting = L.parked || L.pc == PC_DONE;
    if (__all_sync(0xffffffffu, waiting)) {
      if (L.parked) runEvent(L, P, sp);
      if (__all_sync(0xffffffffu, L.pc == PC_DONE)) break;
    }
  }
  if (i < P.n) {
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


} // namespace kfd
