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
//   madd           a*b + c with one renormalisation
// Every step uses the _rn intrinsics so the compiler can neither contract a
// product into a following add nor reorder the sums the algorithms rely on.
// Values must stay inside the float exponent range (about 1e-38..3e38).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

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

// a*b + c without renormalising the product first: the two_prod error terms
// join c's low word before the one renormalisation (15 flops against 18 for
// a separate mul and add; the same "sloppy" error bound)
__device__ __forceinline__ df64 madd(df64 a, df64 b, df64 c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  df64 s = two_sum(p, c.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(e, c.lo));
  return quick_two_sum(s.hi, s.lo);
}
// Four-term sums of the stencil with one renormalisation at the end: the
// high words go through error-free two_sums, the low words and the errors
// are summed as floats ("lazy" double-float accumulation; 27 flops for
// (b+c)-(a+d) against 33 for three renormalised adds).
struct df64_unnorm {
  float hi, lo;  // hi + lo, |lo| not yet bounded by ulp(hi)/2
};
__device__ __forceinline__ df64_unnorm add_lazy(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, b.hi);
  return {s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo))};
}
__device__ __forceinline__ df64 sub_norm(df64_unnorm a, df64_unnorm b) {
  const df64 s = two_sum(a.hi, -b.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df64 add_norm(df64_unnorm a, df64_unnorm b) {
  const df64 s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
// (b + c) - (a + d)
__device__ __forceinline__ df64 diff22(df64 b, df64 c, df64 a, df64 d) {
  return sub_norm(add_lazy(b, c), add_lazy(a, d));
}
// (a + b) + (c + d)
__device__ __forceinline__ df64 sum22(df64 a, df64 b, df64 c, df64 d) {
  return add_norm(add_lazy(a, b), add_lazy(c, d));
}
// (c + d) - (a + b) and (a + b) + (c + d) sharing the pair sums
__device__ __forceinline__ void diffsum22(df64 a, df64 b, df64 c, df64 d, df64 &diff, df64 &sum) {
  const df64_unnorm ab = add_lazy(a, b), cd = add_lazy(c, d);
  diff = sub_norm(cd, ab);
  sum = add_norm(ab, cd);
}
// (b + c) - (a + d) and (c + d) - (a + b) as (c - a) + (b - d) and
// (c - a) - (b - d): two pair differences shared (38 flops against 54)
__device__ __forceinline__ df64_unnorm sub_lazy(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, -b.hi);
  return {s.hi, __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo))};
}
__device__ __forceinline__ void diffdiff22(df64 a, df64 b, df64 c, df64 d, df64 &dx, df64 &dy) {
  const df64_unnorm u = sub_lazy(c, a), w = sub_lazy(b, d);
  dx = add_norm(u, w);
  dy = sub_norm(u, w);
}
template <typename T> __device__ __forceinline__ void diffdiff22(T a, T b, T c, T d, T &dx, T &dy) {
  const T u = c - a, w = b - d;
  dx = u + w;
  dy = u - w;
}
template <typename T> __device__ __forceinline__ T diff22(T b, T c, T a, T d) { return (b + c) - (a + d); }
template <typename T> __device__ __forceinline__ T sum22(T a, T b, T c, T d) { return (a + b) + (c + d); }
template <typename T> __device__ __forceinline__ void diffsum22(T a, T b, T c, T d, T &diff, T &sum) {
  const T ab = a + b, cd = c + d;
  diff = cd - ab;
  sum = ab + cd;
}

// The stencil's pair differences kept unnormalised (lo not yet bounded by
// ulp(hi) / 2) until the add that consumes them renormalises anyway (3 flops
// fewer per value); Lazy<T> is T itself for the native types.
template <typename T> struct Lazy { using type = T; };
template <> struct Lazy<df64> { using type = df64_unnorm; };
__device__ __forceinline__ df64_unnorm sub_unnorm(df64_unnorm a, df64_unnorm b) {
  const df64 s = two_sum(a.hi, -b.hi);
  return {s.hi, __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo))};
}
__device__ __forceinline__ df64_unnorm add_unnorm(df64_unnorm a, df64_unnorm b) {
  const df64 s = two_sum(a.hi, b.hi);
  return {s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo))};
}
__device__ __forceinline__ df64_unnorm diff22_u(df64 b, df64 c, df64 a, df64 d) {
  return sub_unnorm(add_lazy(b, c), add_lazy(a, d));
}
__device__ __forceinline__ df64_unnorm sum22_u(df64 a, df64 b, df64 c, df64 d) {
  return add_unnorm(add_lazy(a, b), add_lazy(c, d));
}
__device__ __forceinline__ void diffsum22_u(df64 a, df64 b, df64 c, df64 d, df64_unnorm &diff, df64_unnorm &sum) {
  const df64_unnorm ab = add_lazy(a, b), cd = add_lazy(c, d);
  diff = sub_unnorm(cd, ab);
  sum = add_unnorm(ab, cd);
}
__device__ __forceinline__ void diffdiff22_u(df64 a, df64 b, df64 c, df64 d, df64_unnorm &dx, df64_unnorm &dy) {
  const df64_unnorm u = sub_lazy(c, a), w = sub_lazy(b, d);
  dx = add_unnorm(u, w);
  dy = sub_unnorm(u, w);
}
__device__ __forceinline__ df64 add_uu(df64_unnorm a, df64_unnorm b) { return add_norm(a, b); }
__device__ __forceinline__ df64 sub_uu(df64_unnorm a, df64_unnorm b) { return sub_norm(a, b); }
__device__ __forceinline__ df64_unnorm to_u(df64 a) { return {a.hi, a.lo}; }
__device__ __forceinline__ df64 norm_u(df64_unnorm a) { return quick_two_sum(a.hi, a.lo); }
template <typename T> __device__ __forceinline__ T diff22_u(T b, T c, T a, T d) { return diff22(b, c, a, d); }
template <typename T> __device__ __forceinline__ T sum22_u(T a, T b, T c, T d) { return sum22(a, b, c, d); }
template <typename T> __device__ __forceinline__ void diffsum22_u(T a, T b, T c, T d, T &diff, T &sum) {
  diffsum22(a, b, c, d, diff, sum);
}
template <typename T> __device__ __forceinline__ void diffdiff22_u(T a, T b, T c, T d, T &dx, T &dy) {
  diffdiff22(a, b, c, d, dx, dy);
}
template <typename T> __device__ __forceinline__ T add_unnorm(T a, T b) { return a + b; }
template <typename T> __device__ __forceinline__ T sub_unnorm(T a, T b) { return a - b; }
template <typename T> __device__ __forceinline__ T add_uu(T a, T b) { return a + b; }
template <typename T> __device__ __forceinline__ T sub_uu(T a, T b) { return a - b; }
template <typename T> __device__ __forceinline__ T to_u(T a) { return a; }
template <typename T> __device__ __forceinline__ T norm_u(T a) { return a; }

// c + sum_j a_j * b_j with one renormalisation at the end (the rows of the
// stiffness product): each product's high part joins the running sum through
// an error-free two_sum, its error terms and the low words are summed as
// floats (12 flops per term against madd's 15, the same "sloppy" bound)
struct df64_acc {
  float hi, lo;
};
__device__ __forceinline__ df64_acc acc_start(df64 c) { return {c.hi, c.lo}; }
__device__ __forceinline__ void acc_madd(df64_acc &s, df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const df64 t = two_sum(s.hi, p);
  s.hi = t.hi;
  s.lo = __fadd_rn(s.lo, __fadd_rn(t.lo, e));
}
__device__ __forceinline__ df64 acc_end(df64_acc s) { return quick_two_sum(s.hi, s.lo); }

// the same for the native types: the compiler contracts a*b + c into one FMA
__device__ __forceinline__ float madd(float a, float b, float c) { return a * b + c; }
__device__ __forceinline__ double madd(double a, double b, double c) { return a * b + c; }

__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }

// ---- between IEEE double and double-float ---------------------------------
// GB300 converts double <-> float on its FP64 unit, at the FP64 FMA rate; these
// conversions run on the integer and FP32 pipes instead (loads) or keep to
// two conversions and one FP64 add (stores).
//
// split_double: d = hi + lo exactly up to the first 47 significant bits (the
// rest truncated: |d - (hi + lo)| < 2^-46 |d|).  hi keeps d's sign, exponent
// and top 23 fraction bits: the double's exponent field, rebiased from 1023
// to 127, is (e11 - 896) mod 256 = (e11 mod 256) ^ 0x80 whenever the result
// is a normal float, so a funnel shift of the high and low words by 3 and a
// flip of bit 30 give hi's bits.  lo holds the next 23 fraction bits m as
// (P | m) - P with P = sign | hi's exponent - 23, exact by Sterbenz.
// Exact (to those 47 bits) for 2^-102 <= |d| < 2^128 (biased exponents
// 921..1150); d == +-0 and every value outside that range give 0 -- the
// double-float path takes only values its range check admitted (see
// in_df64_range), so this only keeps a stray value from becoming garbage.
__device__ __forceinline__ df64 split_double(double d) {
  const uint32_t hw = (uint32_t)__double2hiint(d), lw = (uint32_t)__double2loint(d);
  const uint32_t f = __funnelshift_l(lw, hw, 3) ^ 0x40000000u;
  const uint32_t hib = (f & 0x7fffffffu) | (hw & 0x80000000u);
  const uint32_t pb = (hib & 0xff800000u) - (23u << 23);
  const float lo = __fsub_rn(__uint_as_float(pb | ((lw >> 6) & 0x7fffffu)), __uint_as_float(pb));
  const bool zero = (((hw >> 20) & 0x7ffu) - 921u) > (1150u - 921u);
  return df64(zero ? 0.f : __uint_as_float(hib), zero ? 0.f : lo);
}

// join_double: hi + lo rounded once to the nearest double (both convert
// exactly; the FP64 add rounds the exact sum)
__device__ __forceinline__ double join_double(df64 v) { return __dadd_rn((double)v.hi, (double)v.lo); }

// join_double_int: hi + lo to a double within one unit in the last place,
// on the integer and FP32 pipes (the FP64 unit converts at its FMA rate).
// For a normalised pair (|lo| <= ulp(hi) / 2) the double of hi is its bits
// rebiased (exponent + 896, fraction moved 29 bits down), and lo adds
// k = lo * 2^(52 - E) units of that double's last place (|k| <= 2^28, the 29
// zero bits below hi's fraction: no carry into the exponent).  When hi is a
// power of two and lo of the other sign the sum falls into the binade below,
// whose unit is half as large: k is counted in those units.  k is formed at
// 2^(53 - E) and halved (rounding half up) otherwise.  Zero gives +0; hi below
// 2^-74 (where the scale factor would leave float's range) takes join_double.
__device__ __forceinline__ double join_double_int(df64 v) {
  const uint32_t hb = __float_as_uint(v.hi), lb = __float_as_uint(v.lo);
  const uint32_t u = hb & 0x7fffffffu;
  if (u == 0u) return 0.0;
  const uint32_t e8 = u >> 23;
  if (e8 < 53u) return join_double(v);
  const uint32_t hw = ((u >> 3) + 0x38000000u) | (hb & 0x80000000u);
  const uint32_t lw = hb << 29;
  const int kk = __float2int_rn(__fmul_rn(v.lo, __uint_as_float((307u - e8) << 23)));
  const bool opposite = ((hb ^ lb) & 0x80000000u) != 0u;
  const int mag = abs(kk);
  const int step = ((u & 0x7fffffu) == 0u && opposite) ? mag : (mag + 1) >> 1;
  const long long bits = (long long)(((unsigned long long)hw << 32) | lw) + (opposite ? -step : step);
  return __longlong_as_double(bits);
}

// float_bits_to_double: a normal float's exact double by its bits (exponent
// rebiased by +896, fraction moved 29 bits down); 0 for +-0.  A subnormal
// float (below 2^-126, outside every range the double-float path admits)
// comes out wrong by at most 2^-126.
__device__ __forceinline__ double float_bits_to_double(float f) {
  const uint32_t b = __float_as_uint(f), u = b & 0x7fffffffu;
  const uint32_t hw = u ? (((u >> 3) + 0x38000000u) | (b & 0x80000000u)) : 0u;
  return __hiloint2double((int)hw, (int)(b << 29));
}

// base + (hi + lo): the pair added to a double by two FP64 adds of its exact
// halves (within one unit in the last place of the sum)
__device__ __forceinline__ double add_pair(double base, df64 inc) {
  return __dadd_rn(__dadd_rn(base, float_bits_to_double(inc.hi)), float_bits_to_double(inc.lo));
}

// whether d is 0 or its biased exponent lies in [e_lo, e_hi]: the values the
// double-float path of the FP64 form takes (bounds chosen by the host so that
// every product with the step's coefficients stays within 2^+-100)
__device__ __forceinline__ bool in_df64_range(double d, uint32_t e_lo, uint32_t e_hi) {
  const uint32_t hw = (uint32_t)__double2hiint(d);
  const uint32_t e = (hw >> 20) & 0x7ffu;
  const bool zero = (hw & 0x7fffffffu) == 0u && __double2loint(d) == 0;
  return zero || (e - e_lo) <= (e_hi - e_lo);
}

}  // namespace pn
