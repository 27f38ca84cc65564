// Double-float arithmetic: a value is the unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi) / 2, about 48 significant bits, computed with FP32 instructions only.
//
// Used where the FP32-flux form needs more than FP32 precision (stiffened-gas pressure
// recovery: differences of ~1e9 numbers, divisions by volume fractions down to 1e-8) but not
// the FP64 pipe, which GB300 runs at 1/64 of the FP32 rate.  The building blocks are the
// error-free transformations of Knuth (TwoSum), Dekker (FastTwoSum) and the FMA-based
// TwoProduct; addition, multiplication and division as in the published double-double
// algorithms (Hida, Li and Bailey, "Algorithms for quad-double precision floating point
// arithmetic", 2001), here on FP32 pairs.  Exponent range is FP32's: every quantity held
// this way must stay within about 1e-38..3e38 (energies ~1e11, pressures ~1e10, fractions
// >= 1e-8 here).
#pragma once
#include "ffv_cvt.cuh"

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float a) { return df{a, 0.0f}; }

// the nearest double-float of an FP64 value (the conversions on the integer pipe,
// ffv_cvt.cuh)
__host__ __device__ __forceinline__ df df_from_double(double x) {
  const float h = f32_of_f64(x);
  return df{h, f32_low_of_f64(x, h)};
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return df{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return df{p, __fmaf_rn(a, b, -p)};
}

// addition with the leading parts' error term and the sum of the low parts (the "sloppy"
// double-double addition): its error is below ~2^-46 of the larger operand, the order of the
// pairs' own representation error, at about half the instructions of the variant that
// carries the low parts' error term too
__device__ __forceinline__ df df_add(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ df df_neg(df x) { return df{-x.hi, -x.lo}; }
__device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ df df_add_f(df x, float b) {
  const df s = two_sum(x.hi, b);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, x.lo));
}

__device__ __forceinline__ df df_mul(df x, df y) {
  df p = two_prod(x.hi, y.hi);
  p.lo = __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, p.lo));
  return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ df df_mul_f(df x, float b) {
  df p = two_prod(x.hi, b);
  p.lo = __fmaf_rn(x.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

// x / y: a quotient from the leading parts, corrected once by the remainder x - q y
__device__ __forceinline__ df df_div(df x, df y) {
  const float q1 = __fdiv_rn(x.hi, y.hi);
  const df r = df_sub(x, df_mul_f(y, q1));
  const float q2 = __fdiv_rn(r.hi, y.hi);
  return fast_two_sum(q1, q2);
}

__device__ __forceinline__ float df_to_float(df x) { return __fadd_rn(x.hi, x.lo); }

__device__ __forceinline__ bool df_lt(df x, df y) {
  return x.hi < y.hi || (x.hi == y.hi && x.lo < y.lo);
}
__device__ __forceinline__ bool df_le(df x, df y) {
  return x.hi < y.hi || (x.hi == y.hi && x.lo <= y.lo);
}
__device__ __forceinline__ bool df_isnan(df x) { return isnan(x.hi) || isnan(x.lo); }
