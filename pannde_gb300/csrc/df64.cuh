// df64.cuh -- double-float ("float-float") arithmetic on the FP32 pipes.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// a 48-bit significand.  The operations restate published error-free
// transformations:
//   two_sum        Knuth, TAOCP vol. 2, 4.2.2 (6 flops, exact a+b = s+e)
//   quick_two_sum  Dekker 1971 (3 flops, exact when |a| >= |b|)
//   two_prod       with a fused multiply-add (2 flops, exact a*b = p+e)
//   add            the "sloppy" double-double add of Hida, Li & Bailey,
//                  "Algorithms for quad-double precision floating point
//                  arithmetic" (2001): two_sum of the high words, add the low
//                  words, renormalise (11 flops)
//   mul            two_prod of the high words plus the cross terms, renormalised
// Every step uses the _rn intrinsics so the compiler can neither contract a
// product into a following add nor reorder the sums the algorithms rely on.
// Values must stay inside the float exponent range (about 1e-38..3e38).
#pragma once
#include <cuda_runtime.h>

namespace pn {

struct df64 {
  float hi, lo;
  __device__ __forceinline__ df64() : hi(0.f), lo(0.f) {}
  __device__ __forceinline__ df64(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ explicit df64(float h) : hi(h), lo(0.f) {}
};

__device__ __forceinline__ df64 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df64(s, e);
}

__device__ __forceinline__ df64 quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df64(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }

__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }

__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}

__device__ __forceinline__ df64 &operator+=(df64 &a, df64 b) { return a = a + b; }

__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }

}  // namespace pn
