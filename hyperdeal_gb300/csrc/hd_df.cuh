// hd_df.cuh -- double-word FP32 arithmetic ("FP32x2") for the FP64-storage
// form of the generic advection kernel.
//
// GB300 issues FP32 FMAs at 64 times the rate of FP64 FMAs (1.25 TFLOP/s
// FP64), so the FP64 form of the operator is bound by the FP64 pipe, not by
// HBM.  In FP32x2 mode a value is held as the unevaluated sum hi + lo of two
// floats (about 48 significant bits) and the line contractions run on the
// FP32 pipe:
//   * storage -> FP32x2: the double's sign, exponent and top 23 mantissa bits
//     become `hi` by integer operations (no FP64 instruction); the remaining
//     29 bits, rounded to 23, become `lo` through an exact (Sterbenz)
//     subtraction of two floats of the same binade (the FP32 exponent range
//     bounds the magnitudes: full precision for 2^-103 <= |x| < 2^128);
//   * c * u + acc: the product by the FMA-based TwoProduct (Dekker 1971; the
//     error term of hi*hi is exact, the cross terms hi*lo + lo*hi are added in
//     FP32, lo*lo is dropped), the high parts summed by Knuth's TwoSum (exact),
//     the low parts summed in FP32 -- the "double-word times double-word" and
//     "double-word plus double-word" building blocks of Joldes, Muller and
//     Popescu, "Tight and rigorous error bounds for basic building blocks of
//     double-word arithmetic", ACM TOMS 44 (2017); a sum is renormalised
//     only where it becomes a factor of another product (accumulators that
//     are only added to stay unnormalised);
//   * FP32x2 -> storage: hi and lo become doubles by integer operations and
//     one FP64 add rounds their sum.
// The relative error of a contraction is a few units of 2^-48 of the sum of
// the magnitudes of its terms (FP64: 2^-53); the stage update U + b K is done
// in FP64 on the rounded K, so the solution itself is never truncated.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace hd {

struct f32x2 {
  float hi, lo;
};

// ---- error-free transformations (device, explicitly rounded operations so
// that no multiply-add contraction or reassociation can change them)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// acc += c * u: TwoProduct of the high parts, cross terms in FP32, TwoSum of
// the high parts; the low part of acc is left unnormalised
__device__ __forceinline__ void x2_mac(f32x2& acc, const f32x2& c, const f32x2& u) {
  const float ph = __fmul_rn(c.hi, u.hi);
  float pl = __fmaf_rn(c.hi, u.hi, -ph);
  pl = __fmaf_rn(c.hi, u.lo, pl);
  pl = __fmaf_rn(c.lo, u.hi, pl);
  float s, e;
  two_sum(acc.hi, ph, s, e);
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(e, pl));
}

// c * u as the first term of a sum: x2_mac on a zero accumulator without
// the TwoSum with zero (the same value; a zero product may keep its sign)
__device__ __forceinline__ f32x2 x2_mul(const f32x2& c, const f32x2& u) {
  const float ph = __fmul_rn(c.hi, u.hi);
  float pl = __fmaf_rn(c.hi, u.hi, -ph);
  pl = __fmaf_rn(c.hi, u.lo, pl);
  pl = __fmaf_rn(c.lo, u.hi, pl);
  return f32x2{ph, pl};
}

// hi + lo with |lo| <= ulp(hi) / 2 (TwoSum: valid whatever the magnitudes)
__device__ __forceinline__ f32x2 x2_norm(const f32x2& a) {
  f32x2 r;
  two_sum(a.hi, a.lo, r.hi, r.lo);
  return r;
}

// double -> FP32x2 by integer operations only (no FP64 instruction, and no
// branch that the compiler could turn into predicated FP64 conversions):
//   2^-103 <= |x| < 2^128: hi = x truncated to 24 significant bits, lo = the
//                          rest rounded to 23 bits (relative error <= 2^-47);
//   2^-126 <= |x| < 2^-103: hi as above, lo = 0 (FP32 precision);
//   |x| < 2^-126 (zeros, subnormal doubles, tiny values): signed zero;
//   |x| >= 2^128: signed infinity (NaN stays NaN).
__device__ __forceinline__ f32x2 x2_from_double(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned h = unsigned(b >> 32), l = unsigned(b);
  const unsigned e = (h >> 20) & 0x7FFu;
  const unsigned sgn = h & 0x80000000u;
  const unsigned hn = sgn | ((e - 896u) << 23) | ((h & 0xFFFFFu) << 3) | (l >> 29);
  // base = +-2^(E-23); base + (low 29 bits rounded to 23) in the mantissa
  // field (a carry into the exponent gives exactly 2 * base), minus base
  const unsigned base = sgn | ((e - 919u) << 23);
  const unsigned rb = ((l & 0x1FFFFFFFu) + 32u) >> 6;
  const float lon = __fsub_rn(__uint_as_float(base + rb), __uint_as_float(base));
  const bool normal = e - 897u <= 253u, full = e - 920u <= 230u, big = e > 1150u;
  const bool nan = e == 0x7FFu && ((h & 0xFFFFFu) | l) != 0u;
  const unsigned hb = normal ? hn : big ? (sgn | 0x7F800000u | (nan ? 0x00400000u : 0u)) : sgn;
  f32x2 r;
  r.hi = __uint_as_float(hb);
  r.lo = full ? lon : 0.f;
  return r;
}

// float -> double by integer operations (exact for normal floats and
// infinities/NaN; zeros and subnormal floats give a signed zero)
__device__ __forceinline__ double x2_float_to_double(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned long long sgn = static_cast<unsigned long long>(u & 0x80000000u) << 32;
  const unsigned long long ed = e == 0xFFu ? 0x7FFull : static_cast<unsigned long long>(e + 896u);
  const unsigned long long bits = e == 0u ? sgn : (sgn | (ed << 52) | (static_cast<unsigned long long>(u & 0x7FFFFFu) << 29));
  return __longlong_as_double(static_cast<long long>(bits));
}

// FP32x2 -> double: one FP64 add rounds hi + lo
__device__ __forceinline__ double x2_to_double(const f32x2& a) {
  return __dadd_rn(x2_float_to_double(a.hi), x2_float_to_double(a.lo));
}

// host: exact split of a double coefficient into hi + lo floats
inline f32x2 x2_split_host(double v) {
  f32x2 r;
  r.hi = float(v);
  r.lo = float(v - double(r.hi));
  return r;
}

}  // namespace hd
