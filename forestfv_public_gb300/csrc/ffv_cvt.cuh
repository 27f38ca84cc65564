// FP64 <-> FP32 conversions on the integer pipe.
//
// GB300 executes FP64 arithmetic and the FP64 <-> FP32 conversion instructions at a small
// fraction of its FP32 and integer rates; the FP32-flux form converts every FP64 state
// value it reads and every FP64 value it writes.  These conversions do the IEEE 754
// arithmetic on the bit patterns instead (binary64 -> binary32 rounded to nearest, ties to
// even; binary32 -> binary64 exact), with integer instructions, for normal numbers and
// zeros; every other input (a result below the FP32 normal range, infinities, NaN) takes
// the hardware conversion.  The results are bit-identical to the hardware conversions (a host
// test checks the fast paths against the compiler's conversions).
//
// The functions compile for the host too (with the bit casts done through memcpy), so that
// the test can run them on the CPU.
#pragma once
#include <stdint.h>
#include <string.h>

#ifndef __CUDACC__
#define FFV_CVT_FN static inline
#else
#define FFV_CVT_FN __host__ __device__ __forceinline__
#endif

FFV_CVT_FN uint32_t cvt_hi(double x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__double2hiint(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return (uint32_t)(u >> 32);
#endif
}
FFV_CVT_FN uint32_t cvt_lo(double x) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__double2loint(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return (uint32_t)u;
#endif
}
FFV_CVT_FN double cvt_f64(uint32_t hi, uint32_t lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  const uint64_t u = ((uint64_t)hi << 32) | lo;
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}
FFV_CVT_FN float cvt_f32(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
FFV_CVT_FN uint32_t cvt_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

// (float)x.  binary64: sign, 11-bit exponent biased by 1023, 52-bit mantissa (20 in the high
// word); binary32: sign, 8-bit exponent biased by 127, 23-bit mantissa.  A double with biased
// exponent e in 897..1150 rounds to a normal float of exponent e - 896: its top 23 mantissa
// bits, plus one where the 29 dropped bits exceed half an ulp or equal it with the kept
// mantissa odd.  That carry may run into the exponent, which is the correct rounding (up to
// infinity above the largest float).
FFV_CVT_FN float f32_of_f64(double x) {
  const uint32_t hi = cvt_hi(x), lo = cvt_lo(x);
  const uint32_t e = (hi >> 20) & 0x7FFu;
  if (e - 897u <= 1150u - 897u) {
    const uint32_t m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1FFFFFFFu;
    const uint32_t f = (hi & 0x80000000u) | ((e - 896u) << 23) | m;
    const uint32_t up = (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return cvt_f32(f + up);
  }
  if (((hi & 0x7FFFFFFFu) | lo) == 0u) return cvt_f32(hi & 0x80000000u);
  return (float)x;
}

// (double)f: a normal float's exponent rebiased (+896) and its mantissa shifted up by 29 bits
FFV_CVT_FN double f64_of_f32(float f) {
  const uint32_t u = cvt_bits(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  if (e - 1u <= 253u)
    return cvt_f64((u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3), u << 29);
  if ((u & 0x7FFFFFFFu) == 0u) return cvt_f64(u & 0x80000000u, 0u);
  return (double)f;
}

// x - (double)(f32_of_f64(x)) as a float (rounded to nearest), the low part of x's
// double-float pair, from the dropped mantissa bits: rem units of 2^(e - 1075) when x was
// rounded toward zero, rem - 2^29 of them when it was rounded away, signed as x; converted
// by the integer-to-float instruction and scaled by that power of two.  Inputs with e < 1000
// (|x| < 2^-23) or e > 1149 (where the high part may round to infinity) take FP64
// arithmetic.
FFV_CVT_FN float f32_low_of_f64(double x, float h) {
  const uint32_t hi = cvt_hi(x), lo = cvt_lo(x);
  const uint32_t e = (hi >> 20) & 0x7FFu;
  if (e - 1000u <= 1149u - 1000u) {
    const uint32_t m = lo >> 29;  // the lowest kept mantissa bit is bit 0 of m
    const uint32_t rem = lo & 0x1FFFFFFFu;
    const bool up = rem > 0x10000000u || (rem == 0x10000000u && (m & 1u));
    int32_t r = up ? (int32_t)rem - (int32_t)0x20000000 : (int32_t)rem;
    if (hi & 0x80000000u) r = -r;
    const float scale = cvt_f32((e - 1075u + 127u) << 23);  // 2^(e - 1075), e - 948 >= 52
    return (float)r * scale;
  }
  if (((hi & 0x7FFFFFFFu) | lo) == 0u) return 0.0f;
  return (float)(x - (double)h);
}
