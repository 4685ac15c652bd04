// FP64 values through the FP32 and integer pipes.
//
// GB300 executes FP64 arithmetic and every FP64<->FP32 conversion on a narrow
// pipe (about two operations per clock per SM, against 128 FP32 or integer
// operations), so a kernel that touches each FP64 element with even one such
// instruction is bound by it.  These helpers move FP64 data in and out of
// FP32 arithmetic with integer bit operations instead:
//   split_double   x -> (hi, lo), hi + lo = x to about 2^-47 relative
//   two_sum        s + e = a + b exactly (Knuth's TwoSum, FP32)
//   pair_to_double s + e as an FP64 value, for a TwoSum pair (|e| <= ulp(s))
// Rare inputs (zeros are handled; FP32-denormal or out-of-range magnitudes,
// infinities, NaN) fall back to the FP64 conversions.
#pragma once

#include <cstdint>

namespace mg {

// The rare FP64 fallbacks live in calls so that they stay real branches: an
// if-converted (predicated) FP64 instruction still occupies the FP64 pipe
// for every element, taken or not.
static __device__ __noinline__ float d2f_slow(double x) { return __double2float_rn(x); }
static __device__ __noinline__ double pair_sum_slow(float s, float e) { return (double)s + (double)e; }

// hi = x with its significand truncated to 24 bits (exact in FP32); lo = the
// next 23 significand bits, also exact in FP32.
__device__ __forceinline__ void split_double(double x, float& hi, float& lo) {
  const unsigned int h = (unsigned int)__double2hiint(x), l = (unsigned int)__double2loint(x);
  const unsigned int sign = h & 0x80000000u;
  const int e = (int)((h >> 20) & 0x7ffu);
  const int ef = e - 896;  // FP32 biased exponent of x
  if (ef >= 1 && ef <= 254) {
    hi = __uint_as_float(sign | ((unsigned int)ef << 23) | ((h & 0xfffffu) << 3) | (l >> 29));
    // significand bits 28..6 of x, least significant bit worth 2^(e - 1069)
    const unsigned int r = (l >> 6) & 0x7fffffu;
    const float rf = __uint_as_float(0x4b000000u | r) - 8388608.0f;  // exactly r
    const int es = e - 942;  // FP32 biased exponent of 2^(e - 1069)
    lo = es >= 1 ? rf * __uint_as_float(sign | ((unsigned int)es << 23)) : 0.0f;
  } else if ((h & 0x7fffffffu) == 0u && l == 0u) {
    hi = __uint_as_float(sign);
    lo = 0.0f;
  } else {
    hi = d2f_slow(x);
    lo = 0.0f;
  }
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// s + e for |e| <= ulp(s): the FP64 pattern of s with e added in units of
// 2^-52 of s's binade (e's bits below that unit are dropped).
__device__ __forceinline__ double pair_to_double(float s, float e) {
  const unsigned int sb = __float_as_uint(s), eb = __float_as_uint(e);
  const unsigned int es = (sb >> 23) & 0xffu, ee = (eb >> 23) & 0xffu;
  const int sh = (int)ee - (int)es + 29;  // e's significand shift into s's FP64 units
  if (es == 0u || es == 255u || ee == 255u || sh > 5) return pair_sum_slow(s, e);
  const unsigned int ms = sb & 0x7fffffu;
  unsigned long long d = ((unsigned long long)((sb & 0x80000000u) | ((es + 896u) << 20) | (ms >> 3)) << 32) |
                         ((unsigned long long)(ms & 7u) << 29);
  if (ee != 0u && sh > -24) {
    const unsigned int me = (eb & 0x7fffffu) | 0x800000u;
    unsigned long long n = sh >= 0 ? (unsigned long long)(me << sh) : (unsigned long long)(me >> -sh);
    if ((eb ^ sb) & 0x80000000u) {
      if (ms == 0u) n <<= 1;  // below an exact power of two the unit halves
      d -= n;
    } else {
      d += n;
    }
  }
  return __longlong_as_double((long long)d);
}

}  // namespace mg
