// kf_ff.cuh — float pairs for the mixed form's field values.
//
// A value is carried as hi + lo, two floats (about 48 significant bits),
// built from FP32 instructions with error-free transformations: Knuth's
// two-sum, Dekker's fast two-sum and the FMA two-product (Dekker 1971, "A
// floating-point technique for extending the available precision"; Joldes,
// Muller, Popescu 2017, "Tight and rigorous error bounds for basic building
// blocks of double-word arithmetic").
//
// Use: the mixed form interpolates the FP32 field map on differences from a
// cell corner and adds the corner back exactly as a pair (getFieldFF), so the
// field value that enters the FP64 first RK stage keeps the map's own
// precision instead of one FP32 rounding (3e-8 of B, which moves the fitted
// perigee by ~1e-6 of its resolution on the 30-plane field-map telescope).
// Operations use the _rn intrinsics so that the compiler neither contracts
// nor reorders them.
#pragma once

#include <cuda_runtime.h>

namespace kff {

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff twoSum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ ff fastTwoSum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff twoProd(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ double join(ff x) { return (double)x.hi + (double)x.lo; }

// pair product (error a few 2^-44 relative)
__device__ __forceinline__ ff mul(ff x, ff y) {
  const ff p = twoProd(x.hi, y.hi);
  const float e = __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, p.lo));
  return fastTwoSum(p.hi, e);
}

} // namespace kff
