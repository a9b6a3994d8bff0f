// kf_device.cuh — per-track fitter state machine for sm_103a.
//
// One thread owns one track.  The arithmetic restates the reference
// KalmanFitter hot path (paths relative to the reference project root):
//   EigenStepper::step              Propagator/EigenStepper.ipp:226-332
//   transportMatrix                 Propagator/EigenStepper.ipp:50-124
//   covarianceTransport/boundState  Propagator/detail/CovarianceEngine.hpp:106-371
//   DirectNavigator status/target   Propagator/DirectNavigator.hpp:158-225
//   updateSingleSurfaceStatus       Propagator/detail/SteppingHelper.hpp:31-65
//   ConstrainedStep                 Propagator/ConstrainedStep.hpp:22-108
//   PathLimitReached/SurfaceReached Propagator/StandardAborters.hpp:24-132
//   KalmanFitter actor/aborter      Fitter/KalmanFitter.hpp:216-393, 682-694
//   GainMatrixUpdater               Fitter/GainMatrixUpdater.hpp:34-106
//   GainMatrixSmoother              Fitter/GainMatrixSmoother.hpp:21-94
//   Plane/Line surfaces             Surfaces/detail/PlaneSurface.ipp, LineSurface.ipp
//
// The dense 8x8 and 6x6 products of the reference are evaluated on their
// structural non-zeros only: the RK transport Jacobian is
//   [[I, 0, A, a], [0, 1, 0, b], [0, 0, B, c], [0, 0, 0, 1]]
// (blocks position, time, direction, q/p) and stays in that form under
// multiplication, and the bound-to-bound Jacobian has a zero last column
// except J(5,5) = 1 and a unit row 4.  Skipped terms are exact zeros and ones,
// so the result is the reference's algebra with a different rounding order.
//
// Precision.  Lane<R> carries the transport Jacobians in R.  R = double is
// the plain form (FP64 throughout).  R = float is the mixed form: field
// interpolation in FP32 on differences from a cell corner, RK4 stages k2..k4
// as FP32 offsets from an FP64 k1, the error estimate, the transport matrix
// and all Jacobians in FP32; position, direction, time, step sizes,
// covariance, gain (Joseph-form update) and smoother in FP64.  The mixed form accepts or
// rejects an RK trial on its FP32 error estimate unless that estimate lies
// within 1 % of the tolerance, where the trial is re-evaluated in FP64, so
// its step sequence follows the FP64 fit's.
#pragma once

#include <type_traits>

#include <cfloat>
#include <cstdint>

#include "../../include/gb300kf.h"
#include "kf_adjoint_math.h"
#include "kf_ff.cuh"
#include "kf_material.h"

namespace kfd {

constexpr int kStateStride = 37; // doubles per stored measurement state
// layout of one stored state (smoother input):
//   [0,6) predicted params, [6,12) filtered params, [12,37) bound-to-bound
//   jacobian from the previous state: rows 0..3 cols 0..4 (20) and row 5
//   cols 0..4 (5); the other entries are structural (row 4 = e4, column
//   5 = e5).  The smoother needs no stored covariance (see finalizeSmooth).

struct PlaneD {
  double c[3], U[3], V[3], T[3];
};

struct FieldD {
  int kind;
  int n[3];
  double B[3]; // constant field, scale applied
  double scale;
  double mn[3], invw[3];
  const float4 *grid;
  float Bf[3], mnf[3], invwf[3], scalef; // FP32 copies for the mixed form
  float Blo[3], wf[3], scalelo;          // mixed form: lo parts of B and scale, cell width
};

struct Params {
  int64_t n, stride, wsStride;
  int nSurf;
  int maxSteps, maxTrials, smoothing, faithful;
  double tol, cutoff, mass, overstep, surfTol, outlierCut;
  float tolLoF;         // mixed form: FP32 error estimates up to this accept
  const double *meas;
  const uint64_t *mask;
  const int32_t *nplanes;
  const double *start, *scov, *perigee;
  double *oParams, *oCov, *oChi2, *oSmoothed;
  int32_t *oStatus, *oNMeas, *oNSteps, *oNTrials;
  double *ws;
  int materialEffects;   // kf_config_t.material_effects when the geometry has material
  double *wsCov;         // with material: [S][42][wsStride] predicted and filtered
                         // covariance per state (the general smoother's input)
  const int32_t *perm;   // batched form: queue position -> track index
  int32_t *queueCounter; // batched form: next unclaimed queue position
  FieldD field;
  PlaneD planes[KF_MAX_PLANES];
  kfm::Slab planeSlab[KF_MAX_PLANES]; // surface material (kf_geometry_t.material)
};

// upper-triangle index of (i, j), i <= j, row-major
__host__ __device__ constexpr int ut(int i, int j) {
  return i * 6 - (i * (i - 1)) / 2 + (j - i);
}
__device__ __forceinline__ int sidx(int i, int j) { return i <= j ? ut(i, j) : ut(j, i); }

template <typename T>
__device__ __forceinline__ void cross3(const T a[3], const T b[3], T r[3]) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

// std::max / std::min argument semantics (NaN handling as in the reference)
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }

enum { kAccuracy = 0, kActor = 1, kAborter = 2, kUser = 3 };
enum { kMissed = 0, kReachable = 1, kOnSurface = 2 };
enum { PC_PRE = 0, PC_LOOP = 1, PC_ACT = 2, PC_POST = 3, PC_DONE = 4 };

// ---------------------------------------------------------------------------
// Magnetic field lookup: Test::ConstantBField (Test/Helper.hpp:17-22) or the
// trilinear map (MagneticField/InterpolatedBFieldMap.hpp:178-181), in FP64
// (plain form) or FP32 pairs (mixed form, getFieldFF).
// ---------------------------------------------------------------------------
// (r, z) map (fieldMapperRZ, MagneticField/BFieldMapUtils.cpp:17-136): the
// (br, bz) grid interpolated bilinearly at r = |(x, y)| (in r, then in z), and
// br turned by the position's azimuth (cos phi = x / r, sin phi = y / r; phi =
// 0 on the axis, the reference's transformBField)
static __device__ __forceinline__ void getFieldRZ(const FieldD &F, const double p[3], double B[3]) {
  const double r2 = p[0] * p[0] + p[1] * p[1];
  const double r = sqrt(r2);
  const double gr = (r - F.mn[0]) * F.invw[0], gz = (p[2] - F.mn[2]) * F.invw[2];
  const int ir = min(max((int)floor(gr), 0), F.n[0] - 2);
  const int iz = min(max((int)floor(gz), 0), F.n[2] - 2);
  const double fr = gr - ir, fz = gz - iz;
  const size_t nr = F.n[0], base = (size_t)iz * nr + ir;
  const float4 v00 = __ldg(F.grid + base), v10 = __ldg(F.grid + base + 1);
  const float4 v01 = __ldg(F.grid + base + nr), v11 = __ldg(F.grid + base + nr + 1);
  const double hr = 1 - fr, hz = 1 - fz;
  const double br = ((v00.x * hr + v10.x * fr) * hz + (v01.x * hr + v11.x * fr) * fz) * F.scale;
  const double bz = ((v00.y * hr + v10.y * fr) * hz + (v01.y * hr + v11.y * fr) * fz) * F.scale;
  double cphi = 1., sphi = 0.;
  if (r2 > DBL_MIN) {
    const double inv = 1. / r;
    cphi = p[0] * inv;
    sphi = p[1] * inv;
  }
  B[0] = br * cphi;
  B[1] = br * sphi;
  B[2] = bz;
}

__device__ __forceinline__ void getField(const FieldD &F, const double p[3], double B[3]) {
  if (F.kind == KF_FIELD_CONSTANT) {
    B[0] = F.B[0];
    B[1] = F.B[1];
    B[2] = F.B[2];
    return;
  }
  if (F.kind == KF_FIELD_GRID_RZ) {
    getFieldRZ(F, p, B);
    return;
  }
  int idx[3];
  double f[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double g = (p[a] - F.mn[a]) * F.invw[a];
    int i = (int)floor(g);
    i = min(max(i, 0), F.n[a] - 2);
    idx[a] = i;
    f[a] = g - i;
  }
  const size_t nx = F.n[0], nxy = (size_t)F.n[0] * F.n[1];
  const size_t base = (size_t)idx[2] * nxy + (size_t)idx[1] * nx + idx[0];
  const float4 v000 = __ldg(F.grid + base), v100 = __ldg(F.grid + base + 1);
  const float4 v010 = __ldg(F.grid + base + nx), v110 = __ldg(F.grid + base + nx + 1);
  const float4 v001 = __ldg(F.grid + base + nxy), v101 = __ldg(F.grid + base + nxy + 1);
  const float4 v011 = __ldg(F.grid + base + nxy + nx), v111 = __ldg(F.grid + base + nxy + nx + 1);
  const double gx = 1 - f[0], gy = 1 - f[1], gz = 1 - f[2];
  auto tri = [&](double a000, double a100, double a010, double a110, double a001,
                 double a101, double a011, double a111) {
    double c00 = a000 * gx + a100 * f[0];
    double c10 = a010 * gx + a110 * f[0];
    double c01 = a001 * gx + a101 * f[0];
    double c11 = a011 * gx + a111 * f[0];
    double c0 = c00 * gy + c10 * f[1];
    double c1 = c01 * gy + c11 * f[1];
    return (c0 * gz + c1 * f[2]) * F.scale;
  };
  B[0] = tri(v000.x, v100.x, v010.x, v110.x, v001.x, v101.x, v011.x, v111.x);
  B[1] = tri(v000.y, v100.y, v010.y, v110.y, v001.y, v101.y, v011.y, v111.y);
  B[2] = tri(v000.z, v100.z, v010.z, v110.z, v001.z, v101.z, v011.z, v111.z);
}

// Mixed form: the field as float pairs (kf_ff.cuh).  The cell is found from
// the FP32 position; the weights are taken from the offset to the cell's
// lower corner, p - (min + i w), which is exact for a float-representable
// grid, so they carry no error from the position's magnitude.  The trilinear
// interpolation runs in FP32 on the corner values' differences from the
// lower corner, v - v000, and adds v000 back as a pair: its rounding errors
// scale with the field's variation across the cell, not with the field.
// Mixed form of the (r, z) lookup: weights from the offsets to the cell's
// lower corner, the interpolation on the corner values' differences from the
// lower corner with the corner added back as a pair (as getFieldFF), and the
// azimuth's cosine and sine in FP32
static __device__ __noinline__ void getFieldFFRZ(const FieldD &F, const float p[3], kff::ff B[3]) {
  const float r2 = p[0] * p[0] + p[1] * p[1];
  const float r = sqrtf(r2);
  const float gr = (r - F.mnf[0]) * F.invwf[0], gz = (p[2] - F.mnf[2]) * F.invwf[2];
  const int ir = min(max((int)floorf(gr), 0), F.n[0] - 2);
  const int iz = min(max((int)floorf(gz), 0), F.n[2] - 2);
  const float fr = __fmul_rn(__fsub_rn(r, __fmaf_rn((float)ir, F.wf[0], F.mnf[0])), F.invwf[0]);
  const float fz = __fmul_rn(__fsub_rn(p[2], __fmaf_rn((float)iz, F.wf[2], F.mnf[2])), F.invwf[2]);
  const size_t nr = F.n[0], base = (size_t)iz * nr + ir;
  const float4 v00 = __ldg(F.grid + base), v10 = __ldg(F.grid + base + 1);
  const float4 v01 = __ldg(F.grid + base + nr), v11 = __ldg(F.grid + base + nr + 1);
  const kff::ff sc = {F.scalef, F.scalelo};
  auto bil = [&](float a00, float a10, float a01, float a11) {
    const float d01 = a01 - a00;
    const float c0 = fr * (a10 - a00);
    const float c1 = d01 + fr * ((a11 - a00) - d01);
    return kff::mul(kff::twoSum(a00, c0 + fz * (c1 - c0)), sc);
  };
  const kff::ff br = bil(v00.x, v10.x, v01.x, v11.x);
  B[2] = bil(v00.y, v10.y, v01.y, v11.y);
  float cphi = 1.f, sphi = 0.f;
  if (r2 > FLT_MIN) {
    const float inv = 1.f / r;
    cphi = p[0] * inv;
    sphi = p[1] * inv;
  }
  B[0] = kff::mul(br, {cphi, 0.f});
  B[1] = kff::mul(br, {sphi, 0.f});
}

//
// The position is given as at + inc: `at` an FP32 position (the step's
// start rounded to FP32), inc a small FP32 offset from it (that rounding's
// residual plus the trial increment).  The offset to the corner is formed as
// (at - corner) + inc: at - corner is exact (two FP32 values a few cells
// apart, the corner on the grid), so the weights carry only the rounding of a
// cell-sized number instead of the position's (6e-5 mm at 1 m, which moves
// the fitted d0 by up to 1e-5 of its resolution on the 30-plane map
// telescope).
__device__ __forceinline__ void getFieldFF(const FieldD &F, const float at[3],
                                           const float inc[3], kff::ff B[3]) {
  if (F.kind == KF_FIELD_CONSTANT) {
#pragma unroll
    for (int a = 0; a < 3; ++a) B[a] = {F.Bf[a], F.Blo[a]};
    return;
  }
  if (F.kind == KF_FIELD_GRID_RZ) {
    const float p[3] = {at[0] + inc[0], at[1] + inc[1], at[2] + inc[2]};
    getFieldFFRZ(F, p, B);
    return;
  }
  int idx[3];
  float f[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float g = ((at[a] + inc[a]) - F.mnf[a]) * F.invwf[a];
    int i = (int)floorf(g);
    i = min(max(i, 0), F.n[a] - 2);
    idx[a] = i;
    const float d = __fsub_rn(at[a], __fmaf_rn((float)i, F.wf[a], F.mnf[a]));
    f[a] = __fmul_rn(__fadd_rn(d, inc[a]), F.invwf[a]);
  }
  const size_t nx = F.n[0], nxy = (size_t)F.n[0] * F.n[1];
  const size_t base = (size_t)idx[2] * nxy + (size_t)idx[1] * nx + idx[0];
  const float4 v000 = __ldg(F.grid + base), v100 = __ldg(F.grid + base + 1);
  const float4 v010 = __ldg(F.grid + base + nx), v110 = __ldg(F.grid + base + nx + 1);
  const float4 v001 = __ldg(F.grid + base + nxy), v101 = __ldg(F.grid + base + nxy + 1);
  const float4 v011 = __ldg(F.grid + base + nxy + nx), v111 = __ldg(F.grid + base + nxy + nx + 1);
  const kff::ff sc = {F.scalef, F.scalelo};
  auto tri = [&](float a000, float a100, float a010, float a110, float a001, float a101,
                 float a011, float a111) {
    const float d010 = a010 - a000, d001 = a001 - a000, d011 = a011 - a000;
    const float c00 = f[0] * (a100 - a000);
    const float c10 = d010 + f[0] * ((a110 - a000) - d010);
    const float c01 = d001 + f[0] * ((a101 - a000) - d001);
    const float c11 = d011 + f[0] * ((a111 - a000) - d011);
    const float c0 = c00 + f[1] * (c10 - c00);
    const float c1 = c01 + f[1] * (c11 - c01);
    return kff::mul(kff::twoSum(a000, c0 + f[2] * (c1 - c0)), sc);
  };
  B[0] = tri(v000.x, v100.x, v010.x, v110.x, v001.x, v101.x, v011.x, v111.x);
  B[1] = tri(v000.y, v100.y, v010.y, v110.y, v001.y, v101.y, v011.y, v111.y);
  B[2] = tri(v000.z, v100.z, v010.z, v110.z, v001.z, v101.z, v011.z, v111.z);
}

// ---------------------------------------------------------------------------
// Per-track state
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Cold per-track state: the covariance and the jacToGlobal blocks are read
// and written only at surface events (transport to a surface, filter,
// smoother, final transport), never in the stepping loop.  They live in
// dynamic shared memory, one column per thread ([element][thread]: a warp's
// 32 lanes touch 32 consecutive words, no bank conflicts), so that the
// stepping loop's register set stays small.  Layout for a CTA of n threads:
// cov [21][n], then g03 [12][n] and g46 [6][n], all double.
// ---------------------------------------------------------------------------
constexpr int kLaneSlots = 128; // threads per CTA of the grid form and the adjoint
extern __shared__ __align__(16) unsigned char kfColdSmem[];
template <typename R> __host__ __device__ constexpr size_t coldStateBytes(int threads = kLaneSlots) {
  return (size_t)threads * (21 + 18) * sizeof(double);
}

// Recording hook of a lane: the fit kernels use NoHook (every call compiles
// to nothing); the chi2 adjoint records its tape through these calls.
struct NoHook {
  static constexpr bool kMaterial = false; // surface material code compiled in
  template <class LT> __device__ __forceinline__ void stepBegin(const LT &) {}
  template <class LT> __device__ __forceinline__ void trial(const LT &, double) {}
  template <class LT> __device__ __forceinline__ void stepEnd(const LT &, bool) {}
  template <class LT> __device__ __forceinline__ void actorSet(const LT &, int) {}
  template <class LT> __device__ __forceinline__ void hitBegin(const LT &, int) {}
  __device__ __forceinline__ void hitEnd(bool) {}
};

// the fit kernels for geometries with material (kf_config_t.material_effects):
// the same lane program with the material interaction and the general smoother
// compiled in (the others carry none of that code)
struct MaterialHook : NoHook {
  static constexpr bool kMaterial = true;
};

template <typename R, typename H = NoHook> struct Lane {
  // ---- stepper state (EigenStepper::State)
  double pos[3], dir[3];
  double p, q, t;
  double pathAcc;
  double ss[4]; // ConstrainedStep values
  int ssDir;    // ConstrainedStep direction (+1 / -1)
  int navDir;
  // transport Jacobian blocks.  Plain form: the blocks themselves.  Mixed
  // form: JA and JB hold their offsets from the straight line's, JA - sTr I
  // and JB - I, with sTr the path since the last reset in FP64, so that
  // their FP32 rounding scales with the field's bending, not with the blocks
  // (see applyTransportOffsets and boundStatePlaneMixed).
  R JA[3][3], Ja[3], Jb, JB[3][3], Jc[3];
  double sTr;   // path since the last Jacobian reset (mixed form)
  R k4[3];     // k4 of the last step (derivative rows 4..6)
  bool stepped; // a step since the last Jacobian reset (else derivative = 0)
  // cold state (shared memory, see coldStateBytes)
  __device__ __forceinline__ double &cov(int e) const {
    return reinterpret_cast<double *>(kfColdSmem)[e * blockDim.x + threadIdx.x];
  }
  __device__ __forceinline__ double &g03(int r, int c) const {
    return reinterpret_cast<double *>(kfColdSmem + 21 * sizeof(double) * blockDim.x)[(r * 4 + c) * blockDim.x + threadIdx.x];
  }
  __device__ __forceinline__ double &g46(int r, int c) const {
    return reinterpret_cast<double *>(kfColdSmem + 33 * sizeof(double) * blockDim.x)
        [(r * 2 + c) * blockDim.x + threadIdx.x];
  }
  // per-leg constants (functions of p only)
  double qop, dtds, d37;
  // ---- navigation / actor
  int next, current, nSeq; // current: -1 none, >=0 plane, -2 target line
  int navCache, navCacheSt; // plane and status of the last status() intersection (-1: none)
  long long navCacheLim;    // the path limit (aborter constraint) it was judged against
  uint64_t mask;
  int nHits, measStates, firstPlane;
  bool targetReached, navBreak, smoothed, finished, result, tn, parked;
  int pc, steps, status, rkSteps, rkTrials;
  double chi2;
  double perigee[3];
  int64_t idx;   // track index (inputs and outputs)
  int64_t wsIdx; // workspace column (queue position in the batched form)
  H hook;
};

// ---- ConstrainedStep (ConstrainedStep.hpp:22-108) --------------------------
// min/max/abs comparisons run on an order-preserving integer image of the
// doubles (integer pipe), selecting exactly the values the double comparisons
// select for non-NaN operands.
__device__ __forceinline__ long long okey(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ long long akey(double x) {
  return __double_as_longlong(x) & 0x7fffffffffffffffLL;
}
template <typename R, typename H> __device__ __forceinline__ double ssMax(const Lane<R, H> &L) {
  double m = L.ss[0];
  long long km = okey(m);
#pragma unroll
  for (int i = 1; i < 4; ++i) {
    const long long k = okey(L.ss[i]);
    if (k > km) {
      km = k;
      m = L.ss[i];
    }
  }
  return m;
}
template <typename R, typename H> __device__ __forceinline__ double ssMin(const Lane<R, H> &L) {
  double m = L.ss[0];
  long long km = okey(m);
#pragma unroll
  for (int i = 1; i < 4; ++i) {
    const long long k = okey(L.ss[i]);
    if (k < km) {
      km = k;
      m = L.ss[i];
    }
  }
  return m;
}
template <typename R, typename H> __device__ __forceinline__ double ssValue(const Lane<R, H> &L) {
  return L.ssDir == 1 ? ssMin(L) : ssMax(L);
}
template <typename R, typename H> __device__ __forceinline__ void ssRelease(Lane<R, H> &L, int t) {
  L.ss[t] = (L.ssDir == 1) ? ssMax(L) : ssMin(L);
}
template <typename R, typename H> __device__ __forceinline__ void ssUpdate(Lane<R, H> &L, double v, int t, bool rel) {
  if (rel) ssRelease(L, t);
  const double c = L.ss[t];
  L.ss[t] = akey(c) < akey(v) ? c : v;
}
template <typename R, typename H> __device__ __forceinline__ void ssInit(Lane<R, H> &L, double value) {
  L.ssDir = value > 0. ? 1 : -1;
  L.ss[0] = DBL_MAX * L.ssDir;
  L.ss[1] = DBL_MAX * L.ssDir;
  L.ss[2] = DBL_MAX * L.ssDir;
  L.ss[3] = value;
}

// per-leg constants: q/p, dt/ds and the dt/d(q/p) coefficient
// 1/sqrt(a), a >= 1: an FP32 estimate refined by two Newton-Raphson steps
// y <- y (3 - a y^2) / 2 (each squares the relative error: ~1e-7 -> 1e-14 -> FP64)
__device__ __forceinline__ double rsqrtNewton(double a) {
  double y = (double)rsqrtf((float)a);
  y = y * (1.5 - 0.5 * a * y * y);
  return y * (1.5 - 0.5 * a * y * y);
}

// per-leg constants from 1/p (ip): q/p, dt/ds = sqrt(1 + (m/p)^2) and the
// transport matrix's time-q/p factor m^2 q / (p dt/ds), through one
// 1/sqrt(1 + (m/p)^2) (the reference's hypot and division, EigenStepper.ipp:
// 36-47, :110-112, to an ulp): an FP64 rsqrt in the plain form, an FP32
// estimate refined in FP64 in the mixed form.
template <typename R, typename H>
__device__ __forceinline__ void legConstantsIp(Lane<R, H> &L, double mass, double ip) {
  L.qop = L.q * ip;
  const double x = mass * ip, a = 1. + x * x;
  double y;
  if constexpr (sizeof(R) == sizeof(float)) y = rsqrtNewton(a);
  else y = rsqrt(a);
  L.dtds = a * y;
  L.d37 = mass * mass * L.q * ip * y;
}
template <typename R, typename H> __device__ __forceinline__ void legConstants(Lane<R, H> &L, double mass) {
  legConstantsIp(L, mass, 1. / L.p);
}

// ---- Jacobian resets -------------------------------------------------------
template <typename R, typename H> __device__ __forceinline__ void resetTransport(Lane<R, H> &L) {
  // the mixed form's JB holds JB - I
  constexpr R one = sizeof(R) == sizeof(float) ? R(0) : R(1);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      L.JA[i][j] = R(0);
      L.JB[i][j] = (i == j) ? one : R(0);
    }
    L.Ja[i] = R(0);
    L.Jc[i] = R(0);
  }
  L.Jb = R(0);
  L.sTr = 0.;
  L.stepped = false;
}

// cos and sin of the direction's phi and theta from its components
// (cos theta = z, sin theta = |(x, y)|, cos phi = x / sin theta, ...), with
// 1 / sin theta: shared by the bound Jacobian at a surface and the
// re-initialised jacToGlobal there, which see the same direction
template <typename R> struct DirTrig {
  R cosT, sinT, invS, cosP, sinP;
};
template <typename R, typename H> __device__ __forceinline__ DirTrig<R> dirTrig(const Lane<R, H> &L) {
  DirTrig<R> t;
  const R x = (R)L.dir[0], y = (R)L.dir[1], z = (R)L.dir[2];
  t.cosT = z;
  t.sinT = sqrt(x * x + y * y);
  t.invS = R(1) / t.sinT;
  t.cosP = x * t.invS;
  t.sinP = y * t.invS;
  return t;
}
// FP64 in both forms.  The mixed form takes 1 / sin(theta) from an FP32
// estimate refined by two Newton steps (rsqrtNewton, sin^2 theta is near 1
// on a telescope and bounded away from 0 wherever the bound frame exists)
// instead of the FP64 square root and division.
template <typename R, typename H>
__device__ __forceinline__ DirTrig<double> dirTrigD(const Lane<R, H> &L) {
  DirTrig<double> t;
  const double x = L.dir[0], y = L.dir[1], z = L.dir[2];
  const double s2 = x * x + y * y;
  t.cosT = z;
  if constexpr (sizeof(R) == sizeof(float)) {
    t.invS = rsqrtNewton(s2);
    t.sinT = s2 * t.invS;
  } else {
    t.sinT = sqrt(s2);
    t.invS = 1. / t.sinT;
  }
  t.cosP = x * t.invS;
  t.sinP = y * t.invS;
  return t;
}

// PlaneSurface::initJacobianToGlobal (PlaneSurface.ipp:122-156), in FP64 in
// both forms
template <typename R, typename H>
__device__ __forceinline__ void planeJacToGlobal(Lane<R, H> &L, const PlaneD &pl,
                                                 const DirTrig<double> &tr) {
  const double cosT = tr.cosT, sinT = tr.sinT, cosP = tr.cosP, sinP = tr.sinP;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    L.g03(r, 0) = pl.U[r];
    L.g03(r, 1) = pl.V[r];
    L.g03(r, 2) = 0.;
    L.g03(r, 3) = 0.;
  }
  L.g46(0, 0) = (-sinT) * sinP;
  L.g46(0, 1) = cosT * cosP;
  L.g46(1, 0) = sinT * cosP;
  L.g46(1, 1) = cosT * sinP;
  L.g46(2, 0) = 0.;
  L.g46(2, 1) = (-sinT);
}
template <typename R, typename H> __device__ __forceinline__ void planeJacToGlobal(Lane<R, H> &L, const PlaneD &pl) {
  planeJacToGlobal(L, pl, dirTrigD(L));
}

// LineSurface::referenceFrame (LineSurface.ipp:46-61), line axis z
__device__ __forceinline__ void lineFrame(const double mom[3], double X[3], double Y[3],
                                          double D[3]) {
  Y[0] = 0.;
  Y[1] = 0.;
  Y[2] = 1.;
  double c[3];
  cross3(Y, mom, c);
  const double n = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  X[0] = c[0] / n;
  X[1] = c[1] / n;
  X[2] = c[2] / n;
  cross3(X, Y, D);
}

// ---------------------------------------------------------------------------
// EigenStepper::step (EigenStepper.ipp:226-332)
// ---------------------------------------------------------------------------
template <typename T> struct RkStages {
  T Bf[3], Bm[3], Bl[3], k1[3], k2[3], k3[3], k4[3];
};

// k1 at the current point (evaluatek, EigenStepper.ipp:18-33)
template <typename T>
__device__ __forceinline__ void rkFirst(const FieldD &F, const T pos[3], const T dir[3], T qop,
                                        RkStages<T> &s) {
  getField(F, pos, s.Bf);
  T c[3];
  cross3(dir, s.Bf, c);
#pragma unroll
  for (int i = 0; i < 3; ++i) s.k1[i] = qop * c[i];
}

// tryRungeKuttaStep (EigenStepper.ipp:243-269): k2, k3, k4 and the error
// estimate h^2 |k1 - k2 - k3 + k4|_1
template <typename T>
__device__ __forceinline__ T rkTrial(const FieldD &F, const T pos[3], const T dir[3], T qop, T h,
                                     RkStages<T> &s) {
  const T h2 = h * h, half_h = h * T(0.5);
  T pos1[3], tmp[3], c[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) pos1[i] = pos[i] + half_h * dir[i] + (h2 * T(0.125)) * s.k1[i];
  getField(F, pos1, s.Bm);
#pragma unroll
  for (int i = 0; i < 3; ++i) tmp[i] = dir[i] + half_h * s.k1[i];
  cross3(tmp, s.Bm, c);
#pragma unroll
  for (int i = 0; i < 3; ++i) s.k2[i] = qop * c[i];
#pragma unroll
  for (int i = 0; i < 3; ++i) tmp[i] = dir[i] + half_h * s.k2[i];
  cross3(tmp, s.Bm, c);
#pragma unroll
  for (int i = 0; i < 3; ++i) s.k3[i] = qop * c[i];
  T pos2[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) pos2[i] = pos[i] + h * dir[i] + (h2 * T(0.5)) * s.k3[i];
  getField(F, pos2, s.Bl);
#pragma unroll
  for (int i = 0; i < 3; ++i) tmp[i] = dir[i] + h * s.k3[i];
  cross3(tmp, s.Bl, c);
#pragma unroll
  for (int i = 0; i < 3; ++i) s.k4[i] = qop * c[i];
  const T d0 = s.k1[0] - s.k2[0] - s.k3[0] + s.k4[0];
  const T d1 = s.k1[1] - s.k2[1] - s.k3[1] + s.k4[1];
  const T d2 = s.k1[2] - s.k2[2] - s.k3[2] + s.k4[2];
  const T e = h2 * (fabs(d0) + fabs(d1) + fabs(d2));
  return (e < T(1e-20)) ? T(1e-20) : e;
}

// Mixed form: k1 = q d x B(pos) in FP64 from the paired field value, and
// the other stages as FP32 offsets from it,
//   k2 - k1 = q (d x (Bm - Bf) + h/2 k1 x Bm),  k3 - k1 = q (d x (Bm - Bf) + h/2 k2 x Bm),
//   k4 - k1 = q (d x (Bl - Bf) + h k3 x Bl),
// whose FP32 rounding is relative to the offsets (h kappa and the field's
// change along the step times k), not to k.  The error estimate
// k1 - k2 - k3 + k4 is a sum of offsets; the transport Jacobian takes the
// stages' FP32 values.
struct StagesDelta {
  RkStages<float> s;   // FP32 stages and field values for the transport
  double k1[3];        // k1 in FP64
  kff::ff Bf[3];       // field at the step's start
  float dBm[3], d2[3], d3[3], d4[3];
};

// posf: the step's start rounded to FP32, res: that rounding's residual
__device__ __forceinline__ void rkFirstDelta(const FieldD &F, const float posf[3], const float res[3],
                                             const double dir[3], double qop, StagesDelta &S) {
  getFieldFF(F, posf, res, S.Bf);
  double B[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    B[i] = kff::join(S.Bf[i]);
    S.s.Bf[i] = S.Bf[i].hi;
  }
  double c[3];
  cross3(dir, B, c);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    S.k1[i] = qop * c[i];
    S.s.k1[i] = (float)S.k1[i];
  }
}

// tryRungeKuttaStep (EigenStepper.ipp:243-269) as FP32 offsets from k1; the
// trial positions (pos + res + increment) only locate the field
__device__ __forceinline__ float rkTrialDelta(const FieldD &F, const float pos[3], const float res[3],
                                              const float dir[3], float q, float h, StagesDelta &S) {
  const float h2 = h * h, half_h = h * 0.5f;
  float p1[3], dB[3], a[3], b[3];
  kff::ff B[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) p1[i] = res[i] + half_h * dir[i] + (h2 * 0.125f) * S.s.k1[i];
  getFieldFF(F, pos, p1, B);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    S.s.Bm[i] = B[i].hi;
    dB[i] = (B[i].hi - S.Bf[i].hi) + (B[i].lo - S.Bf[i].lo);
  }
  cross3(dir, dB, a); // d x (Bm - Bf), shared by k2 and k3
  cross3(S.s.k1, S.s.Bm, b);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    S.d2[i] = q * (a[i] + half_h * b[i]);
    S.s.k2[i] = S.s.k1[i] + S.d2[i];
  }
  cross3(S.s.k2, S.s.Bm, b);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    S.d3[i] = q * (a[i] + half_h * b[i]);
    S.s.k3[i] = S.s.k1[i] + S.d3[i];
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) p1[i] = res[i] + h * dir[i] + (h2 * 0.5f) * S.s.k3[i];
  getFieldFF(F, pos, p1, B);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    S.s.Bl[i] = B[i].hi;
    dB[i] = (B[i].hi - S.Bf[i].hi) + (B[i].lo - S.Bf[i].lo);
  }
  cross3(dir, dB, a);
  cross3(S.s.k3, S.s.Bl, b);
  float e = 0.f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    S.d4[i] = q * (a[i] + h * b[i]);
    S.s.k4[i] = S.s.k1[i] + S.d4[i];
    e += fabsf(S.d4[i] - (S.d2[i] + S.d3[i])); // k1 - k2 - k3 + k4
  }
  e *= h2;
  return (e < 1e-20f) ? 1e-20f : e;
}

template <typename R, typename H>
__device__ __forceinline__ void applyTransportStep(Lane<R, H> &L, const R DA[3][3], const R DB[3][3],
                                                   const R Da[3], const R Dc[3], R D37);

// The mixed form's J = D J on offsets from the straight line: with
// A = s I + dA, B = I + dB (the lane's JA, JB), DA = h I + dDA, DB = I + dDB,
//   dA' = dA + h dB + dDA (I + dB),  a' = a + h c + dDA c + Da,
//   dB' = dB + dDB (I + dB),         c' = c + dDB c + Dc,   b' = b + D37,
// every FP32 term a field-induced quantity (the path s is advanced in FP64).
template <typename R, typename H>
__device__ __forceinline__ void applyTransportOffsets(Lane<R, H> &L, R h, const R dDA[3][3],
                                                      const R dDB[3][3], const R Da[3],
                                                      const R Dc[3], R D37) {
  R nA[3][3], na[3], nB[3][3], nc[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const R pA = dDA[i][j] + dDA[i][0] * L.JB[0][j] + dDA[i][1] * L.JB[1][j] + dDA[i][2] * L.JB[2][j];
      const R pB = dDB[i][j] + dDB[i][0] * L.JB[0][j] + dDB[i][1] * L.JB[1][j] + dDB[i][2] * L.JB[2][j];
      nA[i][j] = L.JA[i][j] + (h * L.JB[i][j] + pA);
      nB[i][j] = L.JB[i][j] + pB;
    }
    na[i] = L.Ja[i] + (h * L.Jc[i] + (dDA[i][0] * L.Jc[0] + dDA[i][1] * L.Jc[1] + dDA[i][2] * L.Jc[2] + Da[i]));
    nc[i] = L.Jc[i] + (dDB[i][0] * L.Jc[0] + dDB[i][1] * L.Jc[1] + dDB[i][2] * L.Jc[2] + Dc[i]);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      L.JA[i][j] = nA[i][j];
      L.JB[i][j] = nB[i][j];
    }
    L.Ja[i] = na[i];
    L.Jc[i] = nc[i];
  }
  L.Jb = L.Jb + D37;
}

// transportMatrix (EigenStepper.ipp:50-124) on its non-zero blocks and
// jacTransport = D * jacTransport (EigenStepper.ipp:312-318)
template <typename R, typename H>
__device__ __forceinline__ void transportUpdate(Lane<R, H> &L, const R dir[3], R qop, R h, R d37,
                                                const RkStages<R> &s) {
  const R half_h = h * R(0.5);
  R dk1dL[3], dk2dL[3], dk3dL[3], dk4dL[3], tmp[3], c[3], cc[3];
  cross3(dir, s.Bf, dk1dL);
#pragma unroll
  for (int i = 0; i < 3; ++i) tmp[i] = dir[i] + half_h * s.k1[i];
  cross3(tmp, s.Bm, c);
  cross3(dk1dL, s.Bm, cc);
#pragma unroll
  for (int i = 0; i < 3; ++i) dk2dL[i] = c[i] + (qop * half_h) * cc[i];
#pragma unroll
  for (int i = 0; i < 3; ++i) tmp[i] = dir[i] + half_h * s.k2[i];
  cross3(tmp, s.Bm, c);
  cross3(dk2dL, s.Bm, cc);
#pragma unroll
  for (int i = 0; i < 3; ++i) dk3dL[i] = c[i] + (qop * half_h) * cc[i];
#pragma unroll
  for (int i = 0; i < 3; ++i) tmp[i] = dir[i] + h * s.k3[i];
  cross3(tmp, s.Bl, c);
  cross3(dk3dL, s.Bl, cc);
#pragma unroll
  for (int i = 0; i < 3; ++i) dk4dL[i] = c[i] + (qop * h) * cc[i];
  // dk1dT = qop * [B]x
  R T1[3][3];
  T1[0][0] = R(0);
  T1[0][1] = qop * s.Bf[2];
  T1[0][2] = qop * -s.Bf[1];
  T1[1][0] = qop * -s.Bf[2];
  T1[1][1] = R(0);
  T1[1][2] = qop * s.Bf[0];
  T1[2][0] = qop * s.Bf[1];
  T1[2][1] = qop * -s.Bf[0];
  T1[2][2] = R(0);
  // dk(n+1)dT = qop * colcross(I + hh * dkndT, B)
  R T2[3][3], T3[3][3], T4[3][3];
  auto nextT = [&](const R (&Tp)[3][3], R hh, const R Bx[3], R (&To)[3][3]) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      R col[3], r[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) col[i] = ((i == j) ? R(1) : R(0)) + hh * Tp[i][j];
      cross3(col, Bx, r);
#pragma unroll
      for (int i = 0; i < 3; ++i) To[i][j] = qop * r[i];
    }
  };
  nextT(T1, half_h, s.Bm, T2);
  nextT(T2, half_h, s.Bm, T3);
  nextT(T3, h, s.Bl, T4);
  // D blocks: dFdT (A), dGdT (I + Bd), dFdL (a), dGdL (c), D(3,7).  The
  // mixed form keeps the offsets DA - h I and DB - I (applyTransportOffsets).
  constexpr bool kOffsets = sizeof(R) == sizeof(float);
  const R one = kOffsets ? R(0) : R(1);
  R DA[3][3], DB[3][3], Da[3], Dc[3];
  const R h6 = h / R(6);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      R v = ((i == j) ? one : R(0)) + h6 * (T1[i][j] + T2[i][j] + T3[i][j]);
      DA[i][j] = v * h;
      DB[i][j] = ((i == j) ? one : R(0)) + h6 * (T1[i][j] + R(2) * (T2[i][j] + T3[i][j]) + T4[i][j]);
    }
    Da[i] = (h * h) / R(6) * (dk1dL[i] + dk2dL[i] + dk3dL[i]);
    Dc[i] = h6 * (dk1dL[i] + R(2) * (dk2dL[i] + dk3dL[i]) + dk4dL[i]);
  }
  if constexpr (kOffsets) applyTransportOffsets(L, h, DA, DB, Da, Dc, h * d37);
  else applyTransportStep(L, DA, DB, Da, Dc, h * d37);
}

// new J = D * J on the structured blocks (EigenStepper.ipp:312-318)
template <typename R, typename H>
__device__ __forceinline__ void applyTransportStep(Lane<R, H> &L, const R DA[3][3], const R DB[3][3],
                                                   const R Da[3], const R Dc[3], R D37) {
  // new J = D * J:
  //  A' = A + DA*B,  a' = a + DA*c + Da,  b' = b + D37,
  //  B' = DB*B,      c' = DB*c + Dc
  R nA[3][3], na[3], nB[3][3], nc[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      nA[i][j] = L.JA[i][j] + DA[i][0] * L.JB[0][j] + DA[i][1] * L.JB[1][j] + DA[i][2] * L.JB[2][j];
      nB[i][j] = DB[i][0] * L.JB[0][j] + DB[i][1] * L.JB[1][j] + DB[i][2] * L.JB[2][j];
    }
    na[i] = L.Ja[i] + DA[i][0] * L.Jc[0] + DA[i][1] * L.Jc[1] + DA[i][2] * L.Jc[2] + Da[i];
    nc[i] = DB[i][0] * L.Jc[0] + DB[i][1] * L.Jc[1] + DB[i][2] * L.Jc[2] + Dc[i];
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      L.JA[i][j] = nA[i][j];
      L.JB[i][j] = nB[i][j];
    }
    L.Ja[i] = na[i];
    L.Jc[i] = nc[i];
  }
  L.Jb = L.Jb + D37;
}

template <typename R, typename H> __device__ void rkStep(Lane<R, H> &L, const Params &P) {
  long nTrials = 0;
  double h = ssValue(L);
  if constexpr (sizeof(R) == sizeof(double)) {
    if (P.field.kind == KF_FIELD_CONSTANT) {
      // ---- plain form, uniform field: the same RK4 step and transport matrix
      // through c = d x B and e = c x B (kfa::polyAcceptFwd); the adjoint
      // differentiates these same formulas
      kfa::PolyStep w;
      kfa::polyPrep(L.dir, P.field.B, w);
      L.hook.stepBegin(L);
      for (;;) {
        L.rkTrials++;
        L.hook.trial(L, h);
        kfa::polyCoef(L.qop, h, w);
        if (w.err <= P.tol) break;
        const double scale = smin(smax(0.25, pow(P.tol / fabs(2. * w.err), 0.25)), 4.);
        const double hn = h * scale;
        L.ss[kAccuracy] = hn;
        L.ssDir = hn > 0. ? 1 : -1;
        h = ssValue(L);
        if (h * h < P.cutoff * P.cutoff || nTrials > P.maxTrials) {
          L.hook.stepEnd(L, false);
          return;
        }
        nTrials++;
      }
      L.hook.stepEnd(L, true);
      kfa::PolyOut o;
      kfa::polyAcceptFwd(L.pos, L.dir, L.t, L.qop, h, L.dtds, L.d37, P.field.B, w, o);
      applyTransportStep(L, o.D.DA, o.D.DB, o.D.Da, o.D.Dc, o.D.D37);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        L.pos[i] = o.pos[i];
        L.dir[i] = o.dir[i];
        L.k4[i] = o.k4[i];
      }
      L.t = o.t;
      L.stepped = true;
      L.pathAcc += h;
      L.rkSteps++;
      return;
    }
    // ---- plain form, field map: FP64 stage by stage
    RkStages<double> s;
    rkFirst<double>(P.field, L.pos, L.dir, L.qop, s);
    L.hook.stepBegin(L);
    for (;;) {
      L.rkTrials++;
      L.hook.trial(L, h);
      const double err = rkTrial<double>(P.field, L.pos, L.dir, L.qop, h, s);
      if (err <= P.tol) break;
      const double scale = smin(smax(0.25, pow(P.tol / fabs(2. * err), 0.25)), 4.);
      const double hn = h * scale;
      L.ss[kAccuracy] = hn;
      L.ssDir = hn > 0. ? 1 : -1;
      h = ssValue(L);
      if (h * h < P.cutoff * P.cutoff || nTrials > P.maxTrials) {
        L.hook.stepEnd(L, false);
        return;
      }
      nTrials++;
    }
    L.hook.stepEnd(L, true);
    // propagationTime (EigenStepper.ipp:36-47)
    L.t += h * L.dtds;
    transportUpdate<double>(L, L.dir, L.qop, h, L.d37, s);
    // equations of motion
    const double hh6 = h * h / 6., h6 = h / 6.;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      L.pos[i] = L.pos[i] + (h * L.dir[i] + hh6 * (s.k1[i] + s.k2[i] + s.k3[i]));
      L.dir[i] = L.dir[i] + h6 * (s.k1[i] + 2. * (s.k2[i] + s.k3[i]) + s.k4[i]);
    }
    const double n = sqrt(L.dir[0] * L.dir[0] + L.dir[1] * L.dir[1] + L.dir[2] * L.dir[2]);
    const double inv = 1. / n;
    L.dir[0] *= inv;
    L.dir[1] *= inv;
    L.dir[2] *= inv;
#pragma unroll
    for (int i = 0; i < 3; ++i) L.k4[i] = s.k4[i];
  } else {
    // ---- mixed form: FP32 stage offsets from an FP64 k1, FP32 transport
    const float qopf = (float)L.qop;
    const float posf[3] = {(float)L.pos[0], (float)L.pos[1], (float)L.pos[2]};
    const float res[3] = {(float)(L.pos[0] - (double)posf[0]), (float)(L.pos[1] - (double)posf[1]),
                          (float)(L.pos[2] - (double)posf[2])};
    const float dirf[3] = {(float)L.dir[0], (float)L.dir[1], (float)L.dir[2]};
    const float tolLo = P.tolLoF;
    StagesDelta S;
    rkFirstDelta(P.field, posf, res, L.dir, L.qop, S);
    for (;;) {
      L.rkTrials++;
      const float errf = rkTrialDelta(P.field, posf, res, dirf, qopf, (float)h, S);
      if (errf <= tolLo) break;
      // Not clearly accepted: the FP64 trial decides, and a rejection sets
      // the next trial's size from its error estimate.  The FP32 estimate is
      // a sum of offsets that cancel to ~1 % of their size, good to ~1e-5
      // relative: rescaled from it, the step sizes (the RK partition of the
      // path) would drift from the FP64 fit's by ~3e-6, and a later decision
      // near the tolerance can then go the other way (1e-4 of the perigee's
      // resolution on a few tracks in 1e6).
      RkStages<double> sd;
      rkFirst<double>(P.field, L.pos, L.dir, L.qop, sd);
      const double err = rkTrial<double>(P.field, L.pos, L.dir, L.qop, h, sd);
      if (err <= P.tol) break;
      const double scale = smin(smax(0.25, pow(P.tol / fabs(2. * err), 0.25)), 4.);
      const double hn = h * scale;
      L.ss[kAccuracy] = hn;
      L.ssDir = hn > 0. ? 1 : -1;
      h = ssValue(L);
      if (h * h < P.cutoff * P.cutoff) return;
      if (nTrials > P.maxTrials) return;
      nTrials++;
    }
    L.t += h * L.dtds;
    transportUpdate<float>(L, dirf, qopf, (float)h, (float)L.d37, S.s);
    L.sTr += h;
    // motion: FP64 state, FP64 k1, FP32 sums of the offsets
    //   pos += h d + h^2/6 (3 k1 + d2 + d3),  dir += h/6 (6 k1 + 2 (d2 + d3) + d4)
    const double hh6 = h * h * (1. / 6.), h6 = h * (1. / 6.);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float s23 = S.d2[i] + S.d3[i];
      const float s234 = 2.f * s23 + S.d4[i];
      L.pos[i] = L.pos[i] + (h * L.dir[i] + hh6 * (3. * S.k1[i] + (double)s23));
      L.dir[i] = L.dir[i] + h6 * (6. * S.k1[i] + (double)s234);
    }
    // |dir|^2 = 1 + e with e ~ (h kappa)^2 <= 1e-3: two Newton steps of
    // 1/sqrt from 1 reach FP64 precision (error ~ e^4)
    const double n2 = L.dir[0] * L.dir[0] + L.dir[1] * L.dir[1] + L.dir[2] * L.dir[2];
    double f = 1.5 - 0.5 * n2;
    f = f * (1.5 - 0.5 * n2 * f * f);
    if (fabs(n2 - 1.) > 1e-3) f = 1. / sqrt(n2); // large turning steps
    L.dir[0] *= f;
    L.dir[1] *= f;
    L.dir[2] *= f;
#pragma unroll
    for (int i = 0; i < 3; ++i) L.k4[i] = S.s.k4[i];
  }
  L.stepped = true;
  L.pathAcc += h;
  L.rkSteps++;
}

// ---------------------------------------------------------------------------
// Covariance transport to a surface (CovarianceEngine.hpp:269-290 with
// surfaceDerivative :106-125) on the structural non-zeros.
//   Pt[r][c]  rows 0-2 of jacToGlobal after jacTransport, cols 0..4
//   R3[c]     row 3, cols 0..4 (col 5 is 1)
//   Dd[r][c]  rows 4-6, cols 0..4
// Row 7 is e4 and column 5 is e3 throughout.
// ---------------------------------------------------------------------------
template <typename R> struct Transported {
  R Pt[3][5], R3[5], Dd[3][5];
};

template <typename R, typename H>
__device__ __forceinline__ void applyTransport(const Lane<R, H> &L, Transported<R> &X) {
  // mixed form: JA = sTr I + dA, JB = I + dB (applyTransportOffsets)
  constexpr bool kOffsets = sizeof(R) == sizeof(float);
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    X.Pt[r][0] = (R)L.g03(r, 0);
    X.Pt[r][1] = (R)L.g03(r, 1);
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const R g0 = (R)L.g46(0, c), g1 = (R)L.g46(1, c), g2 = (R)L.g46(2, c);
      const R gr = (R)L.g46(r, c);
      X.Pt[r][2 + c] = (kOffsets ? (R)(L.g03(r, 2 + c) + L.sTr * L.g46(r, c)) : (R)L.g03(r, 2 + c)) +
                       L.JA[r][0] * g0 + L.JA[r][1] * g1 + L.JA[r][2] * g2;
      X.Dd[r][2 + c] = (kOffsets ? gr : R(0)) + L.JB[r][0] * g0 + L.JB[r][1] * g1 + L.JB[r][2] * g2;
    }
    X.Pt[r][4] = L.Ja[r];
    X.Dd[r][0] = R(0);
    X.Dd[r][1] = R(0);
    X.Dd[r][4] = L.Jc[r];
  }
  X.R3[0] = R(0);
  X.R3[1] = R(0);
  X.R3[2] = R(0);
  X.R3[3] = R(0);
  X.R3[4] = L.Jb;
}

// jacToGlobal -= derivative * sVec, then J = jacToLocal * jacToGlobal (in R)
// and cov <- J cov J^T (in FP64).  ax0/ax1 are the surface's local axes
// (rows 0 and 1 of jacToLocal); the direction rows follow
// PlaneSurface.ipp:158-189 / LineSurface.ipp:114-143.
template <typename R, typename H, typename TR>
__device__ __forceinline__ void projectCov(Lane<R, H> &L, Transported<R> &X, const R sVec[5],
                                           const R ax0[3], const R ax1[3], const DirTrig<TR> &tr,
                                           double Jst[25]) {
  // derivative (EigenStepper.ipp:320-325): direction, dt/ds and k4 of the
  // last step; zero right after a Jacobian reset
  R der[7];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    der[r] = L.stepped ? (R)L.dir[r] : R(0);
    der[4 + r] = L.stepped ? L.k4[r] : R(0);
  }
  der[3] = L.stepped ? (R)L.dtds : R(0);
#pragma unroll
  for (int c = 0; c < 5; ++c) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      X.Pt[r][c] -= der[r] * sVec[c];
      X.Dd[r][c] -= der[4 + r] * sVec[c];
    }
    X.R3[c] -= der[3] * sVec[c];
  }
  const R cosT = (R)tr.cosT, sinT = (R)tr.sinT, invS = (R)tr.invS, cosP = (R)tr.cosP,
          sinP = (R)tr.sinP;
  const R j24 = -sinP * invS, j25 = cosP * invS;
  const R j34 = cosP * cosT, j35 = sinP * cosT, j36 = -sinT;
  // the Jacobian's arithmetic type: FP32 in the mixed form (Jacobian
  // transport); the covariance, its transport J C J^T, the gain and the
  // Joseph update are FP64
  using CT = typename std::conditional<sizeof(R) == sizeof(float), float, double>::type;
  CT J[6][6];
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    J[0][c] = ax0[0] * X.Pt[0][c] + ax0[1] * X.Pt[1][c] + ax0[2] * X.Pt[2][c];
    J[1][c] = ax1[0] * X.Pt[0][c] + ax1[1] * X.Pt[1][c] + ax1[2] * X.Pt[2][c];
    J[2][c] = j24 * X.Dd[0][c] + j25 * X.Dd[1][c];
    J[3][c] = j34 * X.Dd[0][c] + j35 * X.Dd[1][c] + j36 * X.Dd[2][c];
    J[4][c] = (c == 4) ? CT(1) : CT(0);
    J[5][c] = X.R3[c];
  }
#pragma unroll
  for (int r = 0; r < 6; ++r) J[r][5] = (r == 5) ? CT(1) : CT(0);
  // C' = J C J^T.  The (loc, angles, q/p) block in FP64 in both forms: the
  // closed-form smoother inverts the same Jacobian, so that block must be
  // J C J^T to well below FP32 rounding (an FP32 product moves the fitted
  // perigee by ~2e-6 of its resolution on the 30-plane field-map telescope).
  // The time row and column (J(i, 5) = 0 for i < 5, so they feed nothing
  // else) in the Jacobian's type.
  double Jd[6][5];
#pragma unroll
  for (int r = 0; r < 6; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) Jd[r][c] = (double)J[r][c];
  // M = J C on rows 0-3, columns 0-4 (row 4 of J is e4)
  double M[4][5];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      double s = Jd[i][0] * L.cov(sidx(0, j));
#pragma unroll
      for (int k = 1; k < 5; ++k) s += Jd[i][k] * L.cov(sidx(k, j));
      M[i][j] = s;
    }
  }
  // time: N = C J(5, :)^T with J(5, 5) = 1, C'(i, 5) = J(i, :) N
  CT N[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    CT s = (CT)L.cov(sidx(k, 5));
#pragma unroll
    for (int l = 0; l < 5; ++l) s += (CT)L.cov(sidx(k, l)) * J[5][l];
    N[k] = s;
  }
  CT T5[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    if (i == 4) {
      T5[4] = N[4];
    } else {
      CT s = (i == 5) ? N[5] : CT(0);
#pragma unroll
      for (int k = 0; k < 5; ++k) s += J[i][k] * N[k];
      T5[i] = s;
    }
  }
  // C' upper triangle
#pragma unroll
  for (int i = 0; i < 5; ++i) {
#pragma unroll
    for (int j = i; j < 5; ++j) {
      double s;
      if (i == 4) {
        s = L.cov(ut(4, 4));
      } else if (j == 4) {
        s = M[i][4];
      } else {
        s = M[i][0] * Jd[j][0];
#pragma unroll
        for (int k = 1; k < 5; ++k) s += M[i][k] * Jd[j][k];
      }
      L.cov(ut(i, j)) = s;
    }
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) L.cov(ut(i, 5)) = (double)T5[i];
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    Jst[c] = Jd[0][c];
    Jst[5 + c] = Jd[1][c];
    Jst[10 + c] = Jd[2][c];
    Jst[15 + c] = Jd[3][c];
    Jst[20 + c] = Jd[5][c];
  }
}

// BoundParameters from the free state (CovarianceEngine.hpp:363-370 and
// coordinate_transformations.hpp:115-128): angles from the momentum
// direction, |p| and q/p as the stepper holds them.  The reference forms q/p
// as charge / |p d| with p = |1 / (q/p)|; with |d| = 1 that is the stepper's
// q/p to an ulp, without the three divisions and the square root.
//
// With absAngles == false the angles are given as offsets from the
// direction's own angles, i.e. 0 (see filterHit).
template <typename R, typename H>
__device__ __forceinline__ void boundAngles(const Lane<R, H> &L, double out[6], double mom[3],
                                            bool absAngles = true) {
#pragma unroll
  for (int i = 0; i < 3; ++i) mom[i] = L.p * L.dir[i];
  if (absAngles) {
    out[2] = atan2(L.dir[1], L.dir[0]);
    out[3] = atan2(sqrt(L.dir[0] * L.dir[0] + L.dir[1] * L.dir[1]), L.dir[2]);
  } else {
    out[2] = 0.;
    out[3] = 0.;
  }
  out[4] = L.qop;
  out[5] = L.t;
}

// 1 / a from an FP32 estimate and two Newton steps y <- y (2 - a y) (each
// squares the relative error), for a of moderate magnitude
__device__ __forceinline__ double rcpNewton(double a) {
  double y = (double)(1.f / (float)a);
  y = y * (2. - a * y);
  return y * (2. - a * y);
}

// C <- J C J^T in FP64 with the bound-to-bound Jacobian J (rows 0-3 and 5,
// columns 0-4; row 4 is e4 and column 5 is e5), on the structural non-zeros,
// and J stored for the smoother (mixed form; projectCov does the same for
// the plain form)
template <typename R, typename H>
__device__ __forceinline__ void transportCovD(Lane<R, H> &L, const double J[6][5], double Jst[25]) {
  double M[4][5];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      double v = J[i][0] * L.cov(sidx(0, j));
#pragma unroll
      for (int k = 1; k < 5; ++k) v += J[i][k] * L.cov(sidx(k, j));
      M[i][j] = v;
    }
  }
  // time: N = C J(5, :)^T with J(5, 5) = 1, C'(i, 5) = J(i, :) N
  double N[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    double v = L.cov(sidx(k, 5));
#pragma unroll
    for (int l = 0; l < 5; ++l) v += L.cov(sidx(k, l)) * J[5][l];
    N[k] = v;
  }
  double T5[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    if (i == 4) {
      T5[4] = N[4];
    } else {
      double v = (i == 5) ? N[5] : 0.;
#pragma unroll
      for (int k = 0; k < 5; ++k) v += J[i][k] * N[k];
      T5[i] = v;
    }
  }
#pragma unroll
  for (int i = 0; i < 5; ++i) {
#pragma unroll
    for (int j = i; j < 5; ++j) {
      double v;
      if (i == 4) {
        v = L.cov(ut(4, 4));
      } else if (j == 4) {
        v = M[i][4];
      } else {
        v = M[i][0] * J[j][0];
#pragma unroll
        for (int k = 1; k < 5; ++k) v += M[i][k] * J[j][k];
      }
      L.cov(ut(i, j)) = v;
    }
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) L.cov(ut(i, 5)) = T5[i];
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    Jst[c] = J[0][c];
    Jst[5 + c] = J[1][c];
    Jst[10 + c] = J[2][c];
    Jst[15 + c] = J[3][c];
    Jst[20 + c] = J[5][c];
  }
}

// boundState<PlaneSurface> in the mixed form (CovarianceEngine.hpp:269-290,
// :106-125; PlaneSurface.ipp:158-204), as the straight line's bound
// Jacobian plus the field-induced remainder.  With JA = s I + dA, JB = I + dB
// the transported jacToGlobal splits into (G03 + s G46, G46), which with
// the derivative term of the direction and the plane's projections gives
// the O(1) entries of J in FP64, and the blocks dA G46, dB G46, Ja, Jc with
// the k4 and dt/ds derivative terms, field-induced, in FP32.  J comes out
// accurate to FP32 rounding of those small terms (an FP32 J moves the fitted
// perigee by up to 3e-6 of its resolution on the 30-plane map telescope,
// mostly through the angle rows), and the covariance transport and the
// smoother take it in FP64.
template <typename H>
__device__ void boundStatePlaneMixed(Lane<float, H> &L, const PlaneD &pl, double out[6],
                                     double Jst[25], bool absAngles) {
  const DirTrig<double> td = dirTrigD(L);
  const double s = L.sTr;
  const bool st = L.stepped;
  // ---- straight-line part, FP64
  const double dp = pl.T[0] * L.dir[0] + pl.T[1] * L.dir[1] + pl.T[2] * L.dir[2];
  const double idp = rcpNewton(dp);
  const double nv[3] = {pl.T[0] * idp, pl.T[1] * idp, pl.T[2] * idp};
  double P0[3][4], s0[4];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) P0[r][c] = L.g03(r, c) + (c >= 2 ? s * L.g46(r, c - 2) : 0.);
#pragma unroll
  for (int c = 0; c < 4; ++c) s0[c] = nv[0] * P0[0][c] + nv[1] * P0[1][c] + nv[2] * P0[2][c];
  if (st) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) P0[r][c] -= L.dir[r] * s0[c];
  }
  const double j24 = -td.sinP * td.invS, j25 = td.cosP * td.invS;
  const double j34 = td.cosP * td.cosT, j35 = td.sinP * td.cosT, j36 = -td.sinT;
  double J[6][5];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    J[0][c] = pl.U[0] * P0[0][c] + pl.U[1] * P0[1][c] + pl.U[2] * P0[2][c];
    J[1][c] = pl.V[0] * P0[0][c] + pl.V[1] * P0[1][c] + pl.V[2] * P0[2][c];
    if (c >= 2) {
      const double g0 = L.g46(0, c - 2), g1 = L.g46(1, c - 2), g2 = L.g46(2, c - 2);
      J[2][c] = j24 * g0 + j25 * g1;
      J[3][c] = j34 * g0 + j35 * g1 + j36 * g2;
    } else {
      J[2][c] = 0.;
      J[3][c] = 0.;
    }
  }
  // ---- field-induced part, FP32
  float G[3][2];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    G[r][0] = (float)L.g46(r, 0);
    G[r][1] = (float)L.g46(r, 1);
  }
  float dP[3][5], dD[3][5];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    dP[r][0] = dP[r][1] = dD[r][0] = dD[r][1] = 0.f;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      dP[r][2 + c] = L.JA[r][0] * G[0][c] + L.JA[r][1] * G[1][c] + L.JA[r][2] * G[2][c];
      dD[r][2 + c] = L.JB[r][0] * G[0][c] + L.JB[r][1] * G[1][c] + L.JB[r][2] * G[2][c];
    }
    dP[r][4] = L.Ja[r];
    dD[r][4] = L.Jc[r];
  }
  const float nvf[3] = {(float)nv[0], (float)nv[1], (float)nv[2]};
  float ds[5], sf[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    ds[c] = nvf[0] * dP[0][c] + nvf[1] * dP[1][c] + nvf[2] * dP[2][c];
    sf[c] = (c < 4 ? (float)s0[c] : 0.f) + ds[c];
  }
  float R3[5];
  if (st) {
    const float d0 = (float)L.dir[0], d1 = (float)L.dir[1], d2 = (float)L.dir[2];
    const float dt = (float)L.dtds;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      dP[0][c] -= d0 * ds[c];
      dP[1][c] -= d1 * ds[c];
      dP[2][c] -= d2 * ds[c];
      dD[0][c] -= L.k4[0] * sf[c];
      dD[1][c] -= L.k4[1] * sf[c];
      dD[2][c] -= L.k4[2] * sf[c];
      R3[c] = (c == 4 ? L.Jb : 0.f) - dt * sf[c];
    }
  } else {
#pragma unroll
    for (int c = 0; c < 5; ++c) R3[c] = (c == 4 ? L.Jb : 0.f);
  }
  const float U[3] = {(float)pl.U[0], (float)pl.U[1], (float)pl.U[2]};
  const float V[3] = {(float)pl.V[0], (float)pl.V[1], (float)pl.V[2]};
  const float f24 = (float)j24, f25 = (float)j25, f34 = (float)j34, f35 = (float)j35, f36 = (float)j36;
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    const float e0 = U[0] * dP[0][c] + U[1] * dP[1][c] + U[2] * dP[2][c];
    const float e1 = V[0] * dP[0][c] + V[1] * dP[1][c] + V[2] * dP[2][c];
    const float e2 = f24 * dD[0][c] + f25 * dD[1][c];
    const float e3 = f34 * dD[0][c] + f35 * dD[1][c] + f36 * dD[2][c];
    if (c < 4) {
      J[0][c] += (double)e0;
      J[1][c] += (double)e1;
      J[2][c] += (double)e2;
      J[3][c] += (double)e3;
    } else {
      J[0][4] = (double)e0;
      J[1][4] = (double)e1;
      J[2][4] = (double)e2;
      J[3][4] = (double)e3;
    }
    J[4][c] = (c == 4) ? 1. : 0.;
    J[5][c] = (double)R3[c];
  }
  transportCovD(L, J, Jst);
  // reinitializeJacobians (CovarianceEngine.hpp:169-201)
  resetTransport(L);
  planeJacToGlobal(L, pl, td);
  const double d0 = L.pos[0] - pl.c[0], d1 = L.pos[1] - pl.c[1], d2 = L.pos[2] - pl.c[2];
  out[0] = pl.U[0] * d0 + pl.U[1] * d1 + pl.U[2] * d2;
  out[1] = pl.V[0] * d0 + pl.V[1] * d1 + pl.V[2] * d2;
  double mom[3];
  boundAngles(L, out, mom, absAngles);
}

// boundState<PlaneSurface> (EigenStepper.ipp:516-540) incl. re-initialisation
template <typename R, typename H>
__device__ void boundStatePlane(Lane<R, H> &L, const PlaneD &pl, double out[6], double Jst[25],
                                bool absAngles = true) {
  if constexpr (sizeof(R) == sizeof(float)) {
    boundStatePlaneMixed(L, pl, out, Jst, absAngles);
    return;
  }
  Transported<R> X;
  applyTransport(L, X);
  // PlaneSurface::derivativeFactors (PlaneSurface.ipp:191-204)
  const R T0 = (R)pl.T[0], T1 = (R)pl.T[1], T2 = (R)pl.T[2];
  const R dp = T0 * (R)L.dir[0] + T1 * (R)L.dir[1] + T2 * (R)L.dir[2];
  const R idp = R(1) / dp;
  const R nv0 = T0 * idp, nv1 = T1 * idp, nv2 = T2 * idp;
  R sVec[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) sVec[c] = nv0 * X.Pt[0][c] + nv1 * X.Pt[1][c] + nv2 * X.Pt[2][c];
  const R U[3] = {(R)pl.U[0], (R)pl.U[1], (R)pl.U[2]};
  const R V[3] = {(R)pl.V[0], (R)pl.V[1], (R)pl.V[2]};
  const DirTrig<double> tr = dirTrigD(L);
  projectCov(L, X, sVec, U, V, tr, Jst);
  // reinitializeJacobians (CovarianceEngine.hpp:169-201)
  resetTransport(L);
  planeJacToGlobal(L, pl, tr);
  const double d0 = L.pos[0] - pl.c[0], d1 = L.pos[1] - pl.c[1], d2 = L.pos[2] - pl.c[2];
  out[0] = pl.U[0] * d0 + pl.U[1] * d1 + pl.U[2] * d2;
  out[1] = pl.V[0] * d0 + pl.V[1] * d1 + pl.V[2] * d2;
  double mom[3];
  boundAngles(L, out, mom, absAngles);
}

// boundState<LineSurface> towards the perigee line (axis z through `c`)
template <typename R, typename H>
__device__ void boundStateLine(Lane<R, H> &L, const double c[3], double out[6]) {
  Transported<R> X;
  applyTransport(L, X);
  double mX[3], mY[3], mD[3];
  lineFrame(L.dir, mX, mY, mD);
  // LineSurface::derivativeFactors (LineSurface.ipp:145-182), locz = (0,0,1)
  const double pc0 = L.pos[0] - c[0], pc1 = L.pos[1] - c[1], pc2 = L.pos[2] - c[2];
  const R rY[3] = {(R)mY[0], (R)mY[1], (R)mY[2]};
  const R rX[3] = {(R)mX[0], (R)mX[1], (R)mX[2]};
  const R dr[3] = {(R)L.dir[0], (R)L.dir[1], (R)L.dir[2]};
  const R long_c = rY[0] * dr[0] + rY[1] * dr[1] + rY[2] * dr[2];
  const R nv0 = dr[0] - long_c * rY[0], nv1 = dr[1] - long_c * rY[1], nv2 = dr[2] - long_c * rY[2];
  const R nrm = R(1) / (R(1) - long_c * long_c);
  const R p0 = (R)pc0, p1 = (R)pc1, p2 = (R)pc2;
  R sVec[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const R s = nv0 * X.Pt[0][k] + nv1 * X.Pt[1][k] + nv2 * X.Pt[2][k];
    const R e0 = rY[0] * s - X.Dd[0][k], e1 = rY[1] * s - X.Dd[1][k], e2 = rY[2] * s - X.Dd[2][k];
    const R row = p0 * e0 + p1 * e1 + p2 * e2;
    sVec[k] = nrm * (s - row);
  }
  double Jst[25];
  projectCov(L, X, sVec, rX, rY, dirTrig(L), Jst);
  double mom[3];
  boundAngles(L, out, mom);
  // LineSurface::globalToLocal (LineSurface.ipp:200-220)
  const double r = sqrt(pc0 * pc0 + pc1 * pc1);
  // (z x mom) . (pos - c)
  const double sgn = ((-mom[1]) * pc0 + mom[0] * pc1 < 0.) ? -1. : 1.;
  out[0] = r * sgn;
  out[1] = pc2;
}

// EigenStepper::update (EigenStepper.ipp:554-564) from bound parameters on a
// plane (boundParameters2freeParameters, coordinate_transformations.hpp:145-158)
template <typename R, typename H>
__device__ __forceinline__ void stepperUpdate(Lane<R, H> &L, const PlaneD &pl, const double par[6],
                                              const double cov[21], double mass) {
#pragma unroll
  for (int r = 0; r < 3; ++r) L.pos[r] = pl.U[r] * par[0] + pl.V[r] * par[1] + pl.c[r];
  double sp, cp, st, ct;
  sincos(par[2], &sp, &cp);
  sincos(par[3], &st, &ct);
  const double d0 = cp * st, d1 = sp * st, d2 = ct;
  const double n2 = d0 * d0 + d1 * d1 + d2 * d2;
  // mixed form: |d|^2 = 1 + O(1e-16), one Newton step of 1/sqrt from 1 is exact
  const double in = (sizeof(R) == sizeof(float)) ? 1.5 - 0.5 * n2 : 1. / sqrt(n2);
  L.dir[0] = d0 * in;
  L.dir[1] = d1 * in;
  L.dir[2] = d2 * in;
  L.p = fabs(1. / par[4]);
  L.t = par[5];
#pragma unroll
  for (int e = 0; e < 21; ++e) L.cov(e) = cov[e];
  legConstantsIp(L, mass, fabs(par[4]));
}

// EigenStepper::update after a filter update whose predicted state is the
// lane's current one.  The filtered angles differ from the predicted ones by
// the gain's correction (the reference evaluates sincos of the filtered
// angles); the predicted angles' cosines and sines are the predicted
// direction's ratios, so the filtered ones follow from the angle-addition
// formulas, with the correction's sine and cosine from Taylor series (|delta|
// <= 0.02: truncation below 1e-20 absolute).  The direction is scaled by
// sin(theta_p) before its normalisation, which removes that division.  Larger
// corrections, and directions within 1e-6 of the z axis, take stepperUpdate.
//
// pred and par may hold the angles as offsets from the predicted direction's
// (absAngles == false); only their difference is used, and the rare
// fallback restores the absolute filtered angles from the direction first.
template <typename R, typename H>
__device__ __forceinline__ void stepperUpdateFiltered(Lane<R, H> &L, const PlaneD &pl,
                                                      const double pred[6], const double par[6],
                                                      const double cov[21], double mass,
                                                      bool absAngles = true) {
  const double dphi = par[2] - pred[2], dth = par[3] - pred[3];
  const double dx = L.dir[0], dy = L.dir[1], dz = L.dir[2];
  const double s2 = dx * dx + dy * dy;
  if (!(fabs(dphi) <= 0.02) || !(fabs(dth) <= 0.02) || !(s2 > 1e-12)) {
    if (absAngles) {
      stepperUpdate(L, pl, par, cov, mass);
    } else {
      double full[6];
#pragma unroll
      for (int e = 0; e < 6; ++e) full[e] = par[e];
      full[2] = atan2(dy, dx) + dphi;
      full[3] = atan2(sqrt(s2), dz) + dth;
      stepperUpdate(L, pl, full, cov, mass);
    }
    return;
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) L.pos[r] = pl.U[r] * par[0] + pl.V[r] * par[1] + pl.c[r];
  auto sinCosSmall = [](double d, double &sn, double &cs) {
    const double d2 = d * d;
    sn = d + d * d2 * (-1. / 6. + d2 * (1. / 120. + d2 * (-1. / 5040.)));
    cs = 1. + d2 * (-0.5 + d2 * (1. / 24. + d2 * (-1. / 720. + d2 * (1. / 40320.))));
  };
  double sdp, cdp, sdt, cdt;
  sinCosSmall(dphi, sdp, cdp);
  sinCosSmall(dth, sdt, cdt);
  // with s = sin(theta_p) = sqrt(s2): cos(phi_p) = dx / s, sin(phi_p) = dy / s,
  // cos(theta_p) = dz; the direction times s
  const double st0 = sqrt(s2);
  const double stf = st0 * cdt + dz * sdt;   // sin(theta_f)
  const double ctf = dz * cdt - st0 * sdt;   // cos(theta_f)
  const double d0 = (dx * cdp - dy * sdp) * stf, d1 = (dy * cdp + dx * sdp) * stf,
               d2 = ctf * st0;
  const double in = rsqrt(d0 * d0 + d1 * d1 + d2 * d2);
  L.dir[0] = d0 * in;
  L.dir[1] = d1 * in;
  L.dir[2] = d2 * in;
  L.p = fabs(1. / par[4]);
  L.t = par[5];
#pragma unroll
  for (int e = 0; e < 21; ++e) L.cov(e) = cov[e];
  legConstantsIp(L, mass, fabs(par[4]));
}

// ---------------------------------------------------------------------------
// Workspace access: state s of track i, element e
// ---------------------------------------------------------------------------
template <typename R, typename H>
__device__ __forceinline__ double *wsPtr(const Params &P, const Lane<R, H> &L, int s, int e) {
  return P.ws + ((size_t)s * kStateStride + e) * (size_t)P.wsStride + L.wsIdx;
}
// with material: predicted (e < 21) and filtered (21 + e) covariance of state s
template <typename R, typename H>
__device__ __forceinline__ double *wsCovPtr(const Params &P, const Lane<R, H> &L, int s, int e) {
  return P.wsCov + ((size_t)s * 42 + e) * (size_t)P.wsStride + L.wsIdx;
}

// ---------------------------------------------------------------------------
// Actor::filter (KalmanFitter.hpp:284-350) for a plane that has a hit, with
// GainMatrixUpdater (GainMatrixUpdater.hpp:34-106).  The plain form keeps the
// reference's (I - KH) C update; the mixed form uses the Joseph form
// (I - KH) C (I - KH)^T + K V K^T, which stays positive definite when the
// predicted covariance carries FP32-level errors from the Jacobian.
// ---------------------------------------------------------------------------
// the material interaction at plane k (material kernels only)
static __device__ __forceinline__ bool materialStep(const Params &P, int k, const double dir[3], double p,
                                          double q, kfm::Effects &fx) {
  return kfm::interact(P.planeSlab[k], P.materialEffects, P.planes[k].T, dir, p, q, P.mass, fx);
}

//
// Angles of the stored states.  The smoother uses a state's angles only in
// x_s = x_f + G (x_s' - x_p') (GainMatrixSmoother.hpp:21-94): as the
// difference of the next state's smoothed and predicted angles, and as this
// state's filtered angle plus a correction.  So a state after the first may
// hold its angles as offsets from its own predicted angles (predicted 0,
// filtered = the gain's correction, smoothed = the smoother's correction):
// the recursion is unchanged and the first state, which keeps absolute
// angles, comes out absolute.  The two atan2 of the predicted angles are
// then evaluated once per track instead of once per surface.  Absolute
// angles stay where a state's angles are read on their own: smoothed states
// returned to the caller, the general smoother with material, the adjoint's
// tape.
template <typename R, typename H>
__device__ void filterHit(Lane<R, H> &L, const Params &P, const PlaneD *planes, int k) {
  const PlaneD &pl = planes[k];
  L.hook.hitBegin(L, k);
  constexpr bool kOffsetForm = std::is_same<H, NoHook>::value;
  const bool absAngles = !kOffsetForm || L.measStates == 0 || P.oSmoothed != nullptr;
  double pred[6], Jst[25];
  boundStatePlane(L, pl, pred, Jst, absAngles);
  const double *mp = P.meas + (size_t)k * 5 * P.stride + L.idx;
  const double m0 = mp[0], m1 = mp[P.stride], v00 = mp[2 * P.stride],
               v01 = mp[3 * P.stride], v11 = mp[4 * P.stride];
  const double S00 = L.cov(0) + v00, S01 = L.cov(1) + v01, S10 = L.cov(1) + v01,
               S11 = L.cov(6) + v11;
  const double det = S00 * S11 - S01 * S10;
  const double idet = 1. / det;
  const double i00 = S11 * idet, i01 = -S01 * idet, i10 = -S10 * idet, i11 = S00 * idet;
  const double r0 = m0 - pred[0], r1 = m1 - pred[1];
  const double chi2 = r0 * (i00 * r0 + i01 * r1) + r1 * (i10 * r0 + i11 * r1);
  const bool outlier = (P.outlierCut > 0. && chi2 > P.outlierCut);
  const int s = L.measStates;
  if (s == 0) L.firstPlane = k;
  // store predicted parameters and the Jacobian
#pragma unroll
  for (int e = 0; e < 6; ++e) *wsPtr(P, L, s, e) = pred[e];
#pragma unroll
  for (int e = 0; e < 25; ++e) *wsPtr(P, L, s, 12 + e) = Jst[e];
  if (H::kMaterial && P.materialEffects) {
    // the general smoother's covariances: predicted, and filtered (= predicted
    // for an outlier, overwritten below otherwise)
    for (int e = 0; e < 21; ++e) {
      *wsCovPtr(P, L, s, e) = L.cov(e);
      *wsCovPtr(P, L, s, 21 + e) = L.cov(e);
    }
  }
  if (outlier) {
    // filtered = predicted; the stepper keeps the predicted state
#pragma unroll
    for (int e = 0; e < 6; ++e) *wsPtr(P, L, s, 6 + e) = pred[e];
  } else {
    double K0[6], K1[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const double c0 = L.cov(sidx(i, 0)), c1 = L.cov(sidx(i, 1));
      K0[i] = c0 * i00 + c1 * i10;
      K1[i] = c0 * i01 + c1 * i11;
    }
    double filt[6], cf[21];
#pragma unroll
    for (int i = 0; i < 6; ++i) filt[i] = pred[i] + (K0[i] * r0 + K1[i] * r1);
    if constexpr (sizeof(R) == sizeof(double)) {
      // the reference's C_f = (I - KH) C (GainMatrixUpdater.hpp:77-84)
#pragma unroll
      for (int i = 0; i < 6; ++i) {
#pragma unroll
        for (int j = i; j < 6; ++j)
          cf[ut(i, j)] = L.cov(ut(i, j)) - K0[i] * L.cov(sidx(0, j)) - K1[i] * L.cov(sidx(1, j));
      }
    } else {
      // Joseph form with H = [I2 0], A = H C (rows 0-1 of C), S = H C H^T + V:
      //   (I - KH) C (I - KH)^T + K V K^T = C - K A - A^T K^T + K S K^T,
      // entry (i, j) = C_ij - K_i . A_j - K_j . (A_i - (K S)_i): four FMAs an
      // entry once D_i = A_i - (K S)_i is formed
      double D0[6], D1[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        D0[i] = L.cov(sidx(0, i)) - (K0[i] * S00 + K1[i] * S10);
        D1[i] = L.cov(sidx(1, i)) - (K0[i] * S01 + K1[i] * S11);
      }
#pragma unroll
      for (int i = 0; i < 6; ++i) {
#pragma unroll
        for (int j = i; j < 6; ++j)
          cf[ut(i, j)] = L.cov(ut(i, j)) - K0[i] * L.cov(sidx(0, j)) - K1[i] * L.cov(sidx(1, j)) -
                         K0[j] * D0[i] - K1[j] * D1[i];
      }
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) *wsPtr(P, L, s, 6 + e) = filt[e];
    if (H::kMaterial && P.materialEffects)
      for (int e = 0; e < 21; ++e) *wsCovPtr(P, L, s, 21 + e) = cf[e];
    L.chi2 += chi2;
    stepperUpdateFiltered(L, pl, pred, filt, cf, P.mass, absAngles);
    if (!P.faithful) planeJacToGlobal(L, pl);
  }
  if constexpr (H::kMaterial) {
    if (P.materialEffects) {
    // the material effects after the filtering (KalmanFitter.hpp:344-345,
    // PointwiseMaterialInteraction.hpp updateState): |p| after the mean energy
    // loss, scattering and Landau variances added to the phi, theta and q/p
    // variances of the bound covariance (an outlier crosses its plane too)
    kfm::Effects fx;
    if (materialStep(P, k, L.dir, L.p, L.q, fx)) {
      L.p = fx.p;
      legConstants(L, P.mass);
      L.cov(ut(2, 2)) = smax(0., L.cov(ut(2, 2)) + fx.varPhi);
      L.cov(ut(3, 3)) = smax(0., L.cov(ut(3, 3)) + fx.varTheta);
      L.cov(ut(4, 4)) = smax(0., L.cov(ut(4, 4)) + fx.varQop);
    }
    }
  }
  L.hook.hitEnd(outlier);
  L.measStates++;
}

// Inverse of the structured bound-to-bound Jacobian
//   J = [[A, b, 0], [0, 1, 0], [c, d, 1]]   (A 4x4, blocks loc/angles, q/p, t)
//   J^-1 = [[A^-1, -A^-1 b, 0], [0, 1, 0], [-c A^-1, -d + c A^-1 b, 1]]
// with A^-1 from its 2x2 blocks (Schur complement).  Output rows 0..3 and 5,
// cols 0..4, in the stored-Jacobian layout.
template <typename T>
__device__ __forceinline__ void invJacobian(const T J[25], T Gi[25]) {
  const T p00 = J[0], p01 = J[1], p10 = J[5], p11 = J[6];
  const T q00 = J[2], q01 = J[3], q10 = J[7], q11 = J[8];
  const T r00 = J[10], r01 = J[11], r10 = J[15], r11 = J[16];
  const T s00 = J[12], s01 = J[13], s10 = J[17], s11 = J[18];
  const T rdp = T(1) / (p00 * p11 - p01 * p10);
  const T i00 = p11 * rdp, i01 = -p01 * rdp, i10 = -p10 * rdp, i11 = p00 * rdp;
  // T = P^-1 Q, U = R P^-1
  const T t00 = i00 * q00 + i01 * q10, t01 = i00 * q01 + i01 * q11;
  const T t10 = i10 * q00 + i11 * q10, t11 = i10 * q01 + i11 * q11;
  const T u00 = r00 * i00 + r01 * i10, u01 = r00 * i01 + r01 * i11;
  const T u10 = r10 * i00 + r11 * i10, u11 = r10 * i01 + r11 * i11;
  // S' = S - R T, Si = S'^-1
  const T a00 = s00 - (r00 * t00 + r01 * t10), a01 = s01 - (r00 * t01 + r01 * t11);
  const T a10 = s10 - (r10 * t00 + r11 * t10), a11 = s11 - (r10 * t01 + r11 * t11);
  const T rds = T(1) / (a00 * a11 - a01 * a10);
  const T z00 = a11 * rds, z01 = -a01 * rds, z10 = -a10 * rds, z11 = a00 * rds;
  T Ai[4][4];
  // lower-right Si, lower-left -Si U, upper-right -T Si, upper-left P^-1 + T Si U
  Ai[2][2] = z00;
  Ai[2][3] = z01;
  Ai[3][2] = z10;
  Ai[3][3] = z11;
  Ai[2][0] = -(z00 * u00 + z01 * u10);
  Ai[2][1] = -(z00 * u01 + z01 * u11);
  Ai[3][0] = -(z10 * u00 + z11 * u10);
  Ai[3][1] = -(z10 * u01 + z11 * u11);
  Ai[0][2] = -(t00 * z00 + t01 * z10);
  Ai[0][3] = -(t00 * z01 + t01 * z11);
  Ai[1][2] = -(t10 * z00 + t11 * z10);
  Ai[1][3] = -(t10 * z01 + t11 * z11);
  Ai[0][0] = i00 - (t00 * Ai[2][0] + t01 * Ai[3][0]);
  Ai[0][1] = i01 - (t00 * Ai[2][1] + t01 * Ai[3][1]);
  Ai[1][0] = i10 - (t10 * Ai[2][0] + t11 * Ai[3][0]);
  Ai[1][1] = i11 - (t10 * Ai[2][1] + t11 * Ai[3][1]);
  const T b[4] = {J[4], J[9], J[14], J[19]};
  const T c[4] = {J[20], J[21], J[22], J[23]};
  const T d = J[24];
  T cb = T(0);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    T v = T(0);
#pragma unroll
    for (int k = 0; k < 4; ++k) v += Ai[r][k] * b[k];
#pragma unroll
    for (int k = 0; k < 4; ++k) Gi[5 * r + k] = Ai[r][k];
    Gi[5 * r + 4] = -v;
    cb += c[r] * v;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    T v = T(0);
#pragma unroll
    for (int r = 0; r < 4; ++r) v += c[r] * Ai[r][k];
    Gi[20 + k] = -v;
  }
  Gi[24] = -d + cb;
}

// ---------------------------------------------------------------------------
// Actor::finalize (KalmanFitter.hpp:360-393) with the gain-matrix (RTS)
// smoother (GainMatrixSmoother.hpp:21-94).  Returns false on a NaN gain.
//
// The reference gain is G = C_f J^T C_p'^-1 with C_p' = J C_f J^T the
// predicted covariance of the next state.  On this path (no material, no
// process noise) that product is exactly J^-1, and the smoothed covariance
// C_s = C_f - G (C_p' - C_s') G^T reduces to G C_s' G^T.  The kernel uses
// these closed forms: the same quantities in exact arithmetic, without the
// cancellation of the reference form (whose q/p variance moves by 1e-9 to
// 5e-8 relative between two valid FP64 evaluations), and without storing
// covariances per state.
// ---------------------------------------------------------------------------
// Smoother when no smoothed-state output is requested: only the first
// state's covariance leaves the fit, C_s(0) = Pg C_f(n-1) Pg^T with
// Pg = G_1 ... G_{n-1} accumulated on the Jacobian structure (~190 instead of
// ~470 FLOP per state for G C_s' G^T).  The gains G_i = J_i^-1 are formed in
// T (FP32 in the mixed form, FP64 in the plain form); the corrections
// J_i^-1 (x_s' - x_p') are FP64-accurate in both: the mixed form refines its
// FP32 product once against the FP64 residual x_s' - x_p' - J_i y.
template <typename T, typename R, typename H>
__device__ bool finalizeSmoothGain(Lane<R, H> &L, const Params &P, const PlaneD *planes) {
  L.smoothed = true;
  const int n = L.measStates;
  double xs[6];
#pragma unroll
  for (int e = 0; e < 6; ++e) xs[e] = *wsPtr(P, L, n - 1, 6 + e);
  T Pg[25];
#pragma unroll
  for (int e = 0; e < 25; ++e) Pg[e] = (e < 20 && e % 6 == 0) ? T(1) : T(0); // rows 0..3: identity
  for (int i = n - 2; i >= 0; --i) {
    T Jn[25], G[25];
#pragma unroll
    for (int e = 0; e < 25; ++e) Jn[e] = (T)*wsPtr(P, L, i + 1, 12 + e);
    invJacobian<T>(Jn, G);
    bool nan = false;
#pragma unroll
    for (int e = 0; e < 25; ++e) nan = nan || (G[e] != G[e]);
    if (nan) return false;
    double dxd[6];
#pragma unroll
    for (int e = 0; e < 6; ++e) dxd[e] = xs[e] - *wsPtr(P, L, i + 1, e);
    // y = G dx on the structure of J^-1
    auto apply = [&](const double v[6], double out[6]) {
      T dx[6];
#pragma unroll
      for (int e = 0; e < 6; ++e) dx[e] = (T)v[e];
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        if (r == 4) {
          out[4] = (double)dx[4];
        } else {
          const int gr = (r == 5) ? 4 : r;
          T g = G[5 * gr] * dx[0];
#pragma unroll
          for (int k = 1; k < 5; ++k) g += G[5 * gr + k] * dx[k];
          if (r == 5) g += dx[5];
          out[r] = (double)g;
        }
      }
    };
    double y[6];
    apply(dxd, y);
    if constexpr (sizeof(T) == sizeof(float)) {
      // FP32 gain: one refinement step with the residual in FP64,
      // r = dx - J y, y += G r, makes y = J^-1 dx to FP64 accuracy
      double rd[6], y1[6];
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        if (r == 4) {
          rd[4] = dxd[4] - y[4];
        } else {
          const int jr = (r == 5) ? 4 : r;
          double v = dxd[r];
#pragma unroll
          for (int k = 0; k < 5; ++k) v -= *wsPtr(P, L, i + 1, 12 + 5 * jr + k) * y[k];
          if (r == 5) v -= y[5];
          rd[r] = v;
        }
      }
      apply(rd, y1);
#pragma unroll
      for (int e = 0; e < 6; ++e) y[e] += y1[e];
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) xs[e] = *wsPtr(P, L, i, 6 + e) + y[e];
    // Pg <- G Pg on the structure [[A, b, 0], [0, 1, 0], [c, d, 1]]
    T Np[25];
#pragma unroll
    for (int r = 0; r < 5; ++r) {
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        T v = G[5 * r] * Pg[c];
#pragma unroll
        for (int k = 1; k < 4; ++k) v += G[5 * r + k] * Pg[5 * k + c];
        if (c == 4) v += G[5 * r + 4];
        if (r == 4) v += Pg[20 + c]; // row 5 of G times row 5 of Pg
        Np[5 * r + c] = v;
      }
    }
#pragma unroll
    for (int e = 0; e < 25; ++e) Pg[e] = Np[e];
  }
  // C_s(0) = Pg C Pg^T with C the last filtered covariance (in the stepper)
  double Cs[21];
  {
    double M[6][6];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        if (r == 4) {
          M[r][c] = L.cov(sidx(4, c));
        } else {
          const int gr = (r == 5) ? 4 : r;
          double v = (double)Pg[5 * gr] * L.cov(sidx(0, c));
#pragma unroll
          for (int k = 1; k < 5; ++k) v += (double)Pg[5 * gr + k] * L.cov(sidx(k, c));
          if (r == 5) v += L.cov(sidx(5, c));
          M[r][c] = v;
        }
      }
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) {
#pragma unroll
      for (int c = r; c < 6; ++c) {
        double v;
        if (c == 4) {
          v = M[r][4];
        } else {
          const int gc = (c == 5) ? 4 : c;
          v = M[r][0] * (double)Pg[5 * gc];
#pragma unroll
          for (int k = 1; k < 5; ++k) v += M[r][k] * (double)Pg[5 * gc + k];
          if (c == 5) v += M[r][5];
        }
        Cs[ut(r, c)] = v;
      }
    }
  }
  const PlaneD &pl = planes[L.firstPlane];
  stepperUpdate(L, pl, xs, Cs, P.mass);
  if (!P.faithful) planeJacToGlobal(L, pl);
  L.navDir = -1;
  ssInit(L, -1. * DBL_MAX);
  L.pathAcc = 0.;
  return true;
}

// ---------------------------------------------------------------------------
// The general gain-matrix smoother (GainMatrixSmoother.hpp:21-94) for fits
// with material noise, where the closed forms above do not hold:
//   G = C_f J^T C_p'^-1,  x_s = x_f + G (x_s' - x_p'),
//   C_s = C_f - G (C_p' - C_s') G^T,
// FP64 in both forms, C_p'^-1 applied through its Cholesky factor.
// ---------------------------------------------------------------------------
// Compiled into the material kernels only (MaterialHook).  u: the track's
// workspace column, i: its track index (outputs), n: states.
static __device__ __forceinline__ bool smoothNoise(const Params &P, int64_t u, int64_t i_, int n,
                                         double xs[6], double Cs[21]) {
  auto WS = [&](int s, int e) { return P.ws[((size_t)s * kStateStride + e) * (size_t)P.wsStride + u]; };
  auto WC = [&](int s, int e) { return P.wsCov[((size_t)s * 42 + e) * (size_t)P.wsStride + u]; };
#pragma unroll
  for (int e = 0; e < 6; ++e) xs[e] = WS(n - 1, 6 + e);
#pragma unroll
  for (int e = 0; e < 21; ++e) Cs[e] = WC(n - 1, 21 + e);
  auto emit = [&](int s) {
    if (!P.oSmoothed) return;
    for (int e = 0; e < 6; ++e) P.oSmoothed[((size_t)s * 27 + e) * P.stride + i_] = xs[e];
    for (int e = 0; e < 21; ++e) P.oSmoothed[((size_t)s * 27 + 6 + e) * P.stride + i_] = Cs[e];
  };
  emit(n - 1);
  for (int i = n - 2; i >= 0; --i) {
    double Cp[21], Cf[21], J[6][6];
#pragma unroll
    for (int e = 0; e < 21; ++e) {
      Cp[e] = WC(i + 1, e);
      Cf[e] = WC(i, 21 + e);
    }
    {
      double Jn[25];
#pragma unroll
      for (int e = 0; e < 25; ++e) Jn[e] = WS(i + 1, 12 + e);
      kfa::jstFull(Jn, J);
    }
    // Cholesky factor of C_p': Lc (lower, row-major upper-triangle layout
    // by (i, j) = ut(j, i)), with the reciprocals of its diagonal
    double Lc[21], id[6];
    bool bad = false;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      double d = Cp[ut(c, c)];
#pragma unroll
      for (int k = 0; k < c; ++k) d -= Lc[ut(k, c)] * Lc[ut(k, c)];
      bad = bad || !(d > 0.);
      const double lcc = sqrt(d);
      id[c] = 1. / lcc;
      Lc[ut(c, c)] = lcc;
#pragma unroll
      for (int r = c + 1; r < 6; ++r) {
        double v = Cp[ut(c, r)];
#pragma unroll
        for (int k = 0; k < c; ++k) v -= Lc[ut(k, r)] * Lc[ut(k, c)];
        Lc[ut(c, r)] = v * id[c];
      }
    }
    if (bad) return false;
    // rows of G: C_p' g = (C_f J^T) row, by forward and back substitution
    double G[6][6];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      // (C_f J^T)(r, c) on J's structure: row 4 is e4, column 5 is e5 (the
      // terms left out are exact zeros)
      double a[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        if (c == 4) {
          a[4] = Cf[sidx(r, 4)];
          continue;
        }
        double v = 0.;
#pragma unroll
        for (int k = 0; k < 5; ++k) v += Cf[sidx(r, k)] * J[c][k];
        if (c == 5) v += Cf[sidx(r, 5)];
        a[c] = v;
      }
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        double v = a[c];
#pragma unroll
        for (int k = 0; k < c; ++k) v -= Lc[ut(k, c)] * a[k];
        a[c] = v * id[c];
      }
#pragma unroll
      for (int c = 5; c >= 0; --c) {
        double v = a[c];
#pragma unroll
        for (int k = c + 1; k < 6; ++k) v -= Lc[ut(c, k)] * a[k];
        a[c] = v * id[c];
      }
      bool nan = false;
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        G[r][c] = a[c];
        nan = nan || (a[c] != a[c]);
      }
      if (nan) return false;
    }
    double xn[6], D[21];
#pragma unroll
    for (int e = 0; e < 6; ++e) {
      double v = 0.;
#pragma unroll
      for (int k = 0; k < 6; ++k) v += G[e][k] * (xs[k] - WS(i + 1, k));
      xn[e] = WS(i, 6 + e) + v;
    }
#pragma unroll
    for (int e = 0; e < 21; ++e) D[e] = Cp[e] - Cs[e];
    double M[6][6];
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        double v = 0.;
#pragma unroll
        for (int k = 0; k < 6; ++k) v += G[r][k] * D[sidx(k, c)];
        M[r][c] = v;
      }
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int c = r; c < 6; ++c) {
        double v = 0.;
#pragma unroll
        for (int k = 0; k < 6; ++k) v += M[r][k] * G[c][k];
        Cs[ut(r, c)] = Cf[ut(r, c)] - v;
      }
#pragma unroll
    for (int e = 0; e < 6; ++e) xs[e] = xn[e];
    emit(i);
  }
  return true;
}

template <typename R, typename H>
__device__ bool finalizeSmooth(Lane<R, H> &L, const Params &P, const PlaneD *planes) {
  L.smoothed = true;
  if (H::kMaterial && P.materialEffects) {
    double xs[6], Cs[21];
    if (!smoothNoise(P, L.wsIdx, L.idx, L.measStates, xs, Cs)) return false;
    const PlaneD &pl = planes[L.firstPlane];
    stepperUpdate(L, pl, xs, Cs, P.mass);
    if (!P.faithful) planeJacToGlobal(L, pl);
    L.navDir = -1;
    ssInit(L, -1. * DBL_MAX);
    L.pathAcc = 0.;
    return true;
  }
  if (!P.oSmoothed) return finalizeSmoothGain<R>(L, P, planes);
  const int n = L.measStates;
  double xs[6], Cs[21];
#pragma unroll
  for (int e = 0; e < 6; ++e) xs[e] = *wsPtr(P, L, n - 1, 6 + e);
  // the stepper holds the last filtered covariance
#pragma unroll
  for (int e = 0; e < 21; ++e) Cs[e] = L.cov(e);
  if (P.oSmoothed) {
#pragma unroll
    for (int e = 0; e < 6; ++e)
      P.oSmoothed[((size_t)(n - 1) * 27 + e) * P.stride + L.idx] = xs[e];
#pragma unroll
    for (int e = 0; e < 21; ++e)
      P.oSmoothed[((size_t)(n - 1) * 27 + 6 + e) * P.stride + L.idx] = Cs[e];
  }
  for (int i = n - 2; i >= 0; --i) {
    double xp[6], Jn[25], xf[6], G[25];
#pragma unroll
    for (int e = 0; e < 6; ++e) xp[e] = *wsPtr(P, L, i + 1, e);
#pragma unroll
    for (int e = 0; e < 25; ++e) Jn[e] = *wsPtr(P, L, i + 1, 12 + e);
#pragma unroll
    for (int e = 0; e < 6; ++e) xf[e] = *wsPtr(P, L, i, 6 + e);
    invJacobian(Jn, G);
    bool nan = false;
#pragma unroll
    for (int e = 0; e < 25; ++e) nan = nan || (G[e] != G[e]);
    if (nan) return false;
    double dx[6];
#pragma unroll
    for (int e = 0; e < 6; ++e) dx[e] = xs[e] - xp[e];
    // rows 0..3 and 5 of G have columns 0..4 stored; row 4 = e4, G(5,5) = 1
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      if (r == 4) {
        xs[4] = xf[4] + dx[4];
      } else {
        const int gr = (r == 5) ? 4 : r;
        double g = G[5 * gr] * dx[0];
#pragma unroll
        for (int k = 1; k < 5; ++k) g += G[5 * gr + k] * dx[k];
        if (r == 5) g += dx[5];
        xs[r] = xf[r] + g;
      }
    }
    // Cs <- G Cs G^T
    double M[6][6];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        if (r == 4) {
          M[r][c] = Cs[sidx(4, c)];
        } else {
          const int gr = (r == 5) ? 4 : r;
          double v = G[5 * gr] * Cs[sidx(0, c)];
#pragma unroll
          for (int k = 1; k < 5; ++k) v += G[5 * gr + k] * Cs[sidx(k, c)];
          if (r == 5) v += Cs[sidx(5, c)];
          M[r][c] = v;
        }
      }
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) {
#pragma unroll
      for (int c = r; c < 6; ++c) {
        double v;
        if (c == 4) {
          v = M[r][4];
        } else {
          const int gc = (c == 5) ? 4 : c;
          v = M[r][0] * G[5 * gc];
#pragma unroll
          for (int k = 1; k < 5; ++k) v += M[r][k] * G[5 * gc + k];
          if (c == 5) v += M[r][5];
        }
        Cs[ut(r, c)] = v;
      }
    }
    if (P.oSmoothed) {
#pragma unroll
      for (int e = 0; e < 6; ++e)
        P.oSmoothed[((size_t)i * 27 + e) * P.stride + L.idx] = xs[e];
#pragma unroll
      for (int e = 0; e < 21; ++e)
        P.oSmoothed[((size_t)i * 27 + 6 + e) * P.stride + L.idx] = Cs[e];
    }
  }
  const PlaneD &pl = planes[L.firstPlane];
  stepperUpdate(L, pl, xs, Cs, P.mass);
  if (!P.faithful) planeJacToGlobal(L, pl);
  L.navDir = -1;
  ssInit(L, -1. * DBL_MAX);
  L.pathAcc = 0.;
  return true;
}

// ---------------------------------------------------------------------------
// Navigation (DirectNavigator.hpp:158-225, SteppingHelper.hpp:31-65)
// ---------------------------------------------------------------------------
template <typename R, typename H>
__device__ __forceinline__ int updateSurfaceStatus(Lane<R, H> &L, const Params &P, const PlaneD &pl,
                                                   int k) {
  const double d0 = L.navDir * L.dir[0], d1 = L.navDir * L.dir[1], d2 = L.navDir * L.dir[2];
  const double denom = d0 * pl.T[0] + d1 * pl.T[1] + d2 * pl.T[2];
  if (denom != 0.0) {
    const double path = (pl.T[0] * (pl.c[0] - L.pos[0]) + pl.T[1] * (pl.c[1] - L.pos[1]) +
                         pl.T[2] * (pl.c[2] - L.pos[2])) /
                        denom;
    if (path * path < P.surfTol * P.surfTol) {
      ssRelease(L, kActor);
      return kOnSurface;
    }
    const double pLimit = L.ss[kAborter];
    const double oLimit = -P.overstep;
    if (path > oLimit && path * path < pLimit * pLimit) {
      ssUpdate(L, L.navDir * path, kActor, true);
      L.hook.actorSet(L, k);
      return kReachable;
    }
  }
  return kMissed;
}

template <typename R, typename H>
__device__ __forceinline__ void navStatus(Lane<R, H> &L, const Params &P, const PlaneD *planes) {
  L.current = -1;
  L.navCache = -1;
  if (L.next != L.nSeq) {
    const int st = updateSurfaceStatus(L, P, planes[L.next], L.next);
    if (st == kOnSurface) {
      L.current = L.next;
      ++L.next;
      if (L.next != L.nSeq) ssRelease(L, kActor);
    } else {
      // target() of the same step asks the same plane from the same state: the
      // state changes between the two only at a surface (never in this branch);
      // the outcome also depends on the path limit, checked at reuse
      L.navCache = L.next;
      L.navCacheSt = st;
      L.navCacheLim = __double_as_longlong(L.ss[kAborter]);
    }
  }
}

template <typename R, typename H>
__device__ __forceinline__ void navTarget(Lane<R, H> &L, const Params &P, const PlaneD *planes) {
  L.current = -1;
  if (L.next != L.nSeq) {
    // the repeated intersection would set the same step constraint again
    const bool reuse = L.navCache == L.next && L.navCacheLim == __double_as_longlong(L.ss[kAborter]);
    const int st = reuse ? L.navCacheSt : updateSurfaceStatus(L, P, planes[L.next], L.next);
    L.navCache = -1;
    if (st == kMissed) ++L.next;
  } else {
    L.navBreak = true;
  }
}

// LineSurface::intersect (LineSurface.ipp:229-262) along navDir * dir
template <typename R, typename H>
__device__ __forceinline__ void lineIntersect(const Lane<R, H> &L, const Params &P, double &u,
                                              int &status) {
  const double ea0 = L.navDir * L.dir[0], ea1 = L.navDir * L.dir[1], ea2 = L.navDir * L.dir[2];
  const double m0 = L.perigee[0] - L.pos[0], m1 = L.perigee[1] - L.pos[1],
               m2 = L.perigee[2] - L.pos[2];
  const double eaTeb = ea2;
  const double denom = 1 - eaTeb * eaTeb;
  if (denom * denom > P.surfTol * P.surfTol) {
    u = ((m0 * ea0 + m1 * ea1 + m2 * ea2) - m2 * eaTeb) / denom;
    status = (u * u < P.surfTol * P.surfTol) ? kOnSurface : kReachable;
  } else {
    u = DBL_MAX;
    status = kMissed;
  }
}

// ---------------------------------------------------------------------------
// The Kalman actor (KalmanFitter.hpp:216-273).  With heavy == false it only
// runs when no filter update, smoothing or final transport is due, and
// returns false without touching the state otherwise.
// ---------------------------------------------------------------------------
template <typename R, typename H>
__device__ bool actor(Lane<R, H> &L, const Params &P, const PlaneD *planes, bool heavy) {
  const bool onPlane = L.current >= 0 && !L.smoothed && !L.finished;
  const bool hit = onPlane && ((L.mask >> L.current) & 1ull);
  if (!heavy) {
    const int ms = L.measStates + (hit ? 1 : 0);
    const bool fin = (ms == L.nHits || (ms > 0 && L.navBreak)) && !L.smoothed && !L.finished &&
                     P.smoothing;
    if (hit || fin) return false;
    if (L.smoothed && !L.finished) {
      if (L.targetReached || L.current == -2) return false;
      double u;
      int st;
      lineIntersect(L, P, u, st);
      if (st == kOnSurface) return false;
    }
  }
  if (hit) filterHit(L, P, planes, L.current);
  if ((L.measStates == L.nHits || (L.measStates > 0 && L.navBreak)) && !L.smoothed &&
      !L.finished) {
    if (!P.smoothing) {
      L.finished = true;
    } else if (!finalizeSmooth(L, P, planes)) {
      L.result = false;
    }
  }
  if (L.smoothed && !L.finished) {
    // SurfaceReached (StandardAborters.hpp:88-132)
    bool reached;
    if (L.targetReached) {
      reached = true;
    } else if (L.current == -2) {
      L.targetReached = true;
      reached = true;
    } else {
      double u;
      int st;
      lineIntersect(L, P, u, st);
      reached = (st == kOnSurface);
      if (reached) {
        L.current = -2;
        L.targetReached = true;
      } else {
        ssUpdate(L, L.navDir * u, kAborter, false);
      }
    }
    if (reached) {
      double out[6];
      boundStateLine(L, L.perigee, out);
#pragma unroll
      for (int e = 0; e < 6; ++e) P.oParams[(size_t)e * P.stride + L.idx] = out[e];
#pragma unroll
      for (int e = 0; e < 21; ++e) P.oCov[(size_t)e * P.stride + L.idx] = L.cov(e);
      L.finished = true;
    }
  }
  return true;
}

// Kalman aborter (KalmanFitter.hpp:682-694) then PathLimitReached
// (StandardAborters.hpp:37-56)
template <typename R, typename H> __device__ __forceinline__ bool aborters(Lane<R, H> &L, const Params &P) {
  if (!L.result || L.finished) return true;
  if (L.targetReached) return true;
  const double distance = L.navDir * fabs(DBL_MAX) - L.pathAcc;
  ssUpdate(L, distance, kAborter, false);
  const bool limit = distance * distance < P.surfTol * P.surfTol;
  if (limit) L.targetReached = true;
  return limit;
}

template <typename R, typename H> __device__ __forceinline__ void finish(Lane<R, H> &L, const Params &P) {
  int st;
  if (!L.result)
    st = L.smoothed ? KF_TRACK_SMOOTHER_NAN : KF_TRACK_MEAS_MISMATCH;
  else if (L.measStates != L.nHits)
    st = KF_TRACK_MEAS_MISMATCH;
  else if (!L.tn)
    st = KF_TRACK_MAX_STEPS;
  else if (P.smoothing && !L.finished)
    st = KF_TRACK_NOT_FITTED;
  else
    st = KF_TRACK_OK;
  L.status = st;
}

// ---------------------------------------------------------------------------
// Propagator::propagate (Propagator.ipp:6-96) as a resumable program:
// advance() runs cheap iterations until the next RK step is done, an event
// (heavy actor work) is due, or the track is done; runEvent() executes the
// pending actor call with heavy work allowed and continues.
// ---------------------------------------------------------------------------
template <typename R, typename H> __device__ void advance(Lane<R, H> &L, const Params &P, const PlaneD *planes) {
  for (;;) {
    switch (L.pc) {
    case PC_PRE:
      if (!actor(L, P, planes, false)) {
        L.parked = true;
        return;
      }
      if (aborters(L, P)) {
        L.pc = PC_POST;
      } else {
        navTarget(L, P, planes);
        L.pc = PC_LOOP;
      }
      continue;
    case PC_LOOP:
      if (L.steps >= P.maxSteps) {
        L.pc = PC_POST;
        continue;
      }
      rkStep(L, P);
      navStatus(L, P, planes);
      L.pc = PC_ACT;
      continue;
    case PC_ACT:
      if (!actor(L, P, planes, false)) {
        L.parked = true;
        return;
      }
      if (aborters(L, P)) {
        L.tn = true;
        L.pc = PC_POST;
        continue;
      }
      navTarget(L, P, planes);
      L.steps++;
      L.pc = PC_LOOP;
      return;
    case PC_POST:
      if (!L.tn) L.navBreak = true;
      if (!actor(L, P, planes, false)) {
        L.parked = true;
        return;
      }
      finish(L, P);
      L.pc = PC_DONE;
      return;
    default:
      return;
    }
  }
}

template <typename R, typename H> __device__ void runEvent(Lane<R, H> &L, const Params &P, const PlaneD *planes) {
  L.parked = false;
  switch (L.pc) {
  case PC_PRE:
    actor(L, P, planes, true);
    if (aborters(L, P)) {
      L.pc = PC_POST;
    } else {
      navTarget(L, P, planes);
      L.pc = PC_LOOP;
    }
    break;
  case PC_ACT:
    actor(L, P, planes, true);
    if (aborters(L, P)) {
      L.tn = true;
      L.pc = PC_POST;
    } else {
      navTarget(L, P, planes);
      L.steps++;
      L.pc = PC_LOOP;
    }
    break;
  case PC_POST:
    actor(L, P, planes, true);
    finish(L, P);
    L.pc = PC_DONE;
    break;
  default:
    break;
  }
}

// EigenStepper::State from BoundParameters<LineSurface> (EigenStepper.hpp:40-61)
// and the navigator initialisation; returns false for unusable input.
template <typename R, typename H>
__device__ void initLane(Lane<R, H> &L, const Params &P, const PlaneD *planes, int64_t i,
                         int64_t wsIdx) {
  L.idx = i;
  L.wsIdx = wsIdx;
  L.pc = PC_DONE;
  L.parked = false;
  L.steps = 0;
  L.rkSteps = 0;
  L.rkTrials = 0;
  L.chi2 = 0.;
  L.measStates = 0;
  L.firstPlane = 0;
  L.next = 0;
  L.current = -1;
  L.navCache = -1;
  L.navCacheSt = 0;
  L.navCacheLim = 0;
  L.targetReached = false;
  L.navBreak = false;
  L.smoothed = false;
  L.finished = false;
  L.result = true;
  L.tn = false;
  L.status = KF_TRACK_NOT_FITTED;
  if (i < 0 || i >= P.n) return;
  double sp[6];
#pragma unroll
  for (int e = 0; e < 6; ++e) sp[e] = P.start[(size_t)e * P.stride + i];
#pragma unroll
  for (int e = 0; e < 3; ++e) L.perigee[e] = P.perigee[(size_t)e * P.stride + i];
  int ns = P.nplanes ? P.nplanes[i] : P.nSurf;
  L.nSeq = min(max(ns, 0), P.nSurf);
  L.mask = P.mask ? P.mask[i] : ~0ull;
  L.nHits = __popcll(L.mask & ((L.nSeq >= 64) ? ~0ull : ((1ull << L.nSeq) - 1ull)));
  bool ok = isfinite(sp[4]) && sp[4] != 0.;
#pragma unroll
  for (int e = 0; e < 6; ++e) ok = ok && isfinite(sp[e]);
  if (!ok) {
    L.status = KF_TRACK_BAD_INPUT;
    return;
  }
  if (L.nHits == 0) {
    L.status = KF_TRACK_NO_HITS;
    return;
  }
  // momentum and position on the line (coordinate_transformations.hpp:45-76,
  // LineSurface.ipp:184-198)
  const double pabs = fabs(1. / sp[4]);
  double sph, cph, sth, cth;
  sincos(sp[2], &sph, &cph);
  sincos(sp[3], &sth, &cth);
  const double mom[3] = {pabs * sth * cph, pabs * sth * sph, pabs * cth};
  const double rad0 = -mom[1], rad1 = mom[0]; // (0,0,1) x mom
  const double rn = sqrt(rad0 * rad0 + rad1 * rad1);
  L.pos[0] = L.perigee[0] + sp[0] * (rad0 / rn);
  L.pos[1] = L.perigee[1] + sp[0] * (rad1 / rn);
  L.pos[2] = (sp[1] + L.perigee[2]) + sp[0] * (0. / rn);
  const double pn = sqrt(mom[0] * mom[0] + mom[1] * mom[1] + mom[2] * mom[2]);
  L.dir[0] = mom[0] / pn;
  L.dir[1] = mom[1] / pn;
  L.dir[2] = mom[2] / pn;
  L.p = pn;
  L.q = (sp[4] > 0) ? 1. : -1.;
  L.t = sp[5];
  L.navDir = 1;
  ssInit(L, DBL_MAX);
  L.pathAcc = 0.;
  resetTransport(L);
#pragma unroll
  for (int e = 0; e < 21; ++e) L.cov(e) = P.scov[(size_t)e * P.stride + i];
  legConstants(L, P.mass);
  // LineSurface::initJacobianToGlobal (LineSurface.ipp:63-112)
  {
    const double x = L.dir[0], y = L.dir[1], z = L.dir[2];
    const double cosT = z, sinT = sqrt(x * x + y * y);
    const double inv = 1. / sinT;
    const double cosP = x * inv, sinP = y * inv;
    double X[3], Y[3], D[3];
    lineFrame(L.dir, X, Y, D);
    double G46[3][2];
    G46[0][0] = (-sinT) * sinP;
    G46[0][1] = cosT * cosP;
    G46[1][0] = sinT * cosP;
    G46[1][1] = cosT * sinP;
    G46[2][0] = 0.;
    G46[2][1] = (-sinT);
    const double ipdn = 1. / (L.dir[0] * D[0] + L.dir[1] * D[1] + L.dir[2] * D[2]);
    double dP[3], dT[3];
    const double cphi[3] = {G46[0][0], G46[1][0], G46[2][0]};
    const double cth_[3] = {G46[0][1], G46[1][1], G46[2][1]};
    cross3(Y, cphi, dP);
    cross3(Y, cth_, dT);
    const double xp = X[0] * dP[0] + X[1] * dP[1] + X[2] * dP[2];
    const double xt = X[0] * dT[0] + X[1] * dT[1] + X[2] * dT[2];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      dP[r] = dP[r] - xp * X[r];
      dT[r] = dT[r] - xt * X[r];
      L.g03(r, 0) = (R)X[r];
      L.g03(r, 1) = (R)Y[r];
      L.g03(r, 2) = (R)(dP[r] * sp[0] * ipdn);
      L.g03(r, 3) = (R)(dT[r] * sp[0] * ipdn);
      L.g46(r, 0) = (R)G46[r][0];
      L.g46(r, 1) = (R)G46[r][1];
    }
  }
  L.pc = PC_PRE;
  navStatus(L, P, planes);
}

} // namespace kfd
