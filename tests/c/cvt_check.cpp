// Host check of the integer-pipe FP64 <-> FP32 conversions (ffv_cvt.cuh) against the
// compiler's own conversions: random bit patterns over the whole exponent range, ties, the
// edges of the FP32 normal range, zeros, subnormals, infinities and NaN.  Prints the number
// of mismatches of each function and exits nonzero if there is any.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "ffv_cvt.cuh"

static uint64_t state = 0x2545F4914F6CDD1Dull;
static uint64_t next_u64() {
  state ^= state << 13;
  state ^= state >> 7;
  state ^= state << 17;
  return state;
}
static double dbl(uint64_t u) {
  double x;
  memcpy(&x, &u, 8);
  return x;
}
static uint32_t fbits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}
static uint64_t dbits(double x) {
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
}

static long bad_hi = 0, bad_lo = 0, bad_up = 0, checked = 0;

static void check_double(double x) {
  checked++;
  const float ref = (float)x, got = f32_of_f64(x);
  if (!(std::isnan(ref) && std::isnan(got)) && fbits(ref) != fbits(got)) {
    if (bad_hi < 5) printf("f32_of_f64(%a): %a, expected %a\n", x, got, ref);
    bad_hi++;
  }
  if (std::isfinite(ref)) {
    const float lref = (float)(x - (double)ref), lgot = f32_low_of_f64(x, ref);
    if (fbits(lref) != fbits(lgot)) {
      if (bad_lo < 5) printf("f32_low_of_f64(%a): %a, expected %a\n", x, lgot, lref);
      bad_lo++;
    }
  }
}

static void check_float(float f) {
  const double ref = (double)f, got = f64_of_f32(f);
  if (!(std::isnan(ref) && std::isnan(got)) && dbits(ref) != dbits(got)) {
    if (bad_up < 5) printf("f64_of_f32(%a): %a, expected %a\n", (double)f, got, ref);
    bad_up++;
  }
}

int main() {
  // random patterns: every exponent, random mantissas and signs
  for (long i = 0; i < 4000000; i++) check_double(dbl(next_u64()));
  // exponents around the FP32 range and the typical magnitudes of the state
  for (long i = 0; i < 4000000; i++) {
    const uint64_t u = next_u64();
    const uint64_t e = 860 + (u >> 52) % 320;  // biased exponents 860..1179
    check_double(dbl((u & 0x800FFFFFFFFFFFFFull) | (e << 52)));
  }
  // ties and near-ties of the 29 dropped bits, both parities of the kept mantissa
  const uint32_t tails[] = {0x10000000u, 0x0FFFFFFFu, 0x10000001u, 0x1FFFFFFFu, 0u, 1u};
  for (long i = 0; i < 200000; i++) {
    const uint64_t u = next_u64();
    const uint64_t e = 890 + (u >> 52) % 270;
    for (uint32_t t : tails) {
      const uint64_t v = (u & 0x800FFFFFE0000000ull) | (e << 52) | t;
      check_double(dbl(v));
    }
  }
  // zeros, subnormals, the edges of the FP32 range, infinities, NaN
  const double specials[] = {0.0, -0.0, 5e-324, -5e-324, 1e-310, 1.1754943508222875e-38,
                             1.1754942106924411e-38, 1.401298464324817e-45, 7e-46,
                             3.4028234663852886e+38, 3.4028235677973366e+38, 3.4028236e+38,
                             -3.4028235677973366e+38, 1e300, -1e300, INFINITY, -INFINITY, NAN,
                             1.0, -1.0, 0.1, 1e-8, 6e8, 5e10};
  for (double x : specials) check_double(x);
  for (long i = 0; i < 4000000; i++) {
    uint32_t u = (uint32_t)next_u64();
    float f;
    memcpy(&f, &u, 4);
    check_float(f);
  }
  const float fspecials[] = {0.0f, -0.0f, 1e-45f, -1e-45f, 1e-40f, 1.17549435e-38f,
                             3.40282347e+38f, INFINITY, -INFINITY, NAN, 1.0f, -2.5f};
  for (float f : fspecials) check_float(f);
  printf("checked %ld doubles: f32_of_f64 %ld mismatches, f32_low_of_f64 %ld; f64_of_f32 %ld\n",
         checked, bad_hi, bad_lo, bad_up);
  return (bad_hi || bad_lo || bad_up) ? 1 : 0;
}
