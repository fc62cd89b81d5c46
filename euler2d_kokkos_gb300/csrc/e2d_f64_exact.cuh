// e2d_f64_exact.cuh -- exact FP64 operations carried out on the integer
// pipe.
//
// GB300 issues FP64 arithmetic at ~1.7 operations per SM per clock, about
// 1/70 of its FP32 rate.  Comparisons, min/max against known signs, sign
// tests and multiplications by 0.5 or 2 do not need the FP64 unit: on the
// bit patterns of IEEE-754 doubles they are integer operations that give the
// same bits as the FP64 instructions.  Each helper states the inputs for which
// that holds; outside them (NaN, subnormal results) it falls back to the FP64
// instruction itself, so results stay bit-identical to the plain expression.
#pragma once

#include <cuda_runtime.h>

namespace e2d {
namespace f64x {

constexpr unsigned long long kMag = 0x7fffffffffffffffull;
constexpr unsigned long long kSign = 0x8000000000000000ull;

__device__ __forceinline__ long long sbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ unsigned long long ubits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ double from_bits(unsigned long long b) {
  return __longlong_as_double((long long)b);
}

// FP64 multiply kept out of line so that it runs only on the lanes that need
// it (a branch, not a predicated instruction issued by the whole warp).
static __device__ __noinline__ double mul_slow(double a, double b) { return a * b; }

// fmax(x, c) for c > 0: non-negative doubles order like their bit patterns as
// signed integers and every negative x (including -0) is below c.
// (NaN x is returned instead of c; NaN states are flagged elsewhere.)
__device__ __forceinline__ double max_pos(double x, double c) { return sbits(x) > sbits(c) ? x : c; }

// fmax / fmin of two non-negative doubles.
__device__ __forceinline__ double max_nn(double a, double b) { return sbits(a) > sbits(b) ? a : b; }
__device__ __forceinline__ double min_nn(double a, double b) { return sbits(a) < sbits(b) ? a : b; }

// fmin / fmax of two doubles of any sign: the key flips the magnitude bits of
// negatives so that keys order like the values; -0 orders below +0 (either
// is a valid fmin(+0, -0)).
__device__ __forceinline__ long long okey(double x) {
  const long long b = sbits(x);
  return b ^ ((b >> 63) & (long long)kMag);
}
__device__ __forceinline__ double min_any(double a, double b) { return okey(a) <= okey(b) ? a : b; }
__device__ __forceinline__ double max_any(double a, double b) { return okey(a) >= okey(b) ? a : b; }

// Sign tests for non-NaN x.
__device__ __forceinline__ bool gt0(double x) { return sbits(x) > 0; }   // x > 0.0
__device__ __forceinline__ bool le0(double x) { return sbits(x) <= 0; }  // x <= 0.0

// 0.5 * x: decrement the exponent of normal numbers with a biased exponent in
// [2, 2046]; zeros are unchanged; subnormal results need rounding and use the
// FP64 multiply; Inf/NaN are unchanged.
__device__ __forceinline__ double half(double x) {
  const int hi = __double2hiint(x);
  const int lo = __double2loint(x);
  const int e = (hi >> 20) & 0x7ff;
  if (e >= 2 && e < 0x7ff) return __hiloint2double(hi - 0x00100000, lo);
  if (((hi & 0x7fffffff) | lo) == 0 || e == 0x7ff) return x;
  return mul_slow(0.5, x);
}

// 2.0 * x: increment the exponent of normal numbers below 2^1023 ...; zeros
// unchanged; subnormals and overflow use the FP64 multiply.
__device__ __forceinline__ double twice(double x) {
  const int hi = __double2hiint(x);
  const int lo = __double2loint(x);
  const int e = (hi >> 20) & 0x7ff;
  if (e >= 1 && e < 0x7fe) return __hiloint2double(hi + 0x00100000, lo);
  if (((hi & 0x7fffffff) | lo) == 0 || e == 0x7ff) return x;
  return mul_slow(2.0, x);
}

static __device__ __noinline__ bool product_le0_slow(double a, double b) { return (a * b) <= 0.0; }

// src/HydroBaseFunctor.h:421-455, one direction, for slope_type st in {1, 2}:
//   dlft = st*(q-qm); drgt = st*(qp-q); dcen = 0.5*(qp-qm)
//   dsgn = dcen >= 0 ? 1 : -1; slop = fmin(|dlft|, |drgt|)
//   dlim = (dlft*drgt <= 0) ? 0 : slop;  dq = dsgn * fmin(dlim, |dcen|)
// The three differences are FP64; scaling by st and 0.5 is exact, min of
// non-negative values and all sign logic are integer operations.  The product
// test dlft*drgt <= 0 equals "a zero or opposite signs" unless the product
// underflows to zero, which needs both magnitudes below 2^-511: that case is
// decided by the FP64 product itself.
__device__ __forceinline__ double slope_limited(bool st2, double q, double qp, double qm) {
  const double d1 = q - qm;
  const double d2 = qp - q;
  const double dc = qp - qm;
  const long long b1 = sbits(d1), b2 = sbits(d2);
  const unsigned long long a1 = (unsigned long long)b1 & kMag;
  const unsigned long long a2 = (unsigned long long)b2 & kMag;
  bool kill = (a1 == 0ull) | (a2 == 0ull) | ((b1 ^ b2) < 0);
  constexpr unsigned long long kTiny = 512ull << 52;  // 2^-511
  if (!kill && (a1 < kTiny || a2 < kTiny)) {
    const double st = st2 ? 2.0 : 1.0;
    kill = product_le0_slow(mul_slow(st, d1), mul_slow(st, d2));
  }
  const unsigned long long m = a1 < a2 ? a1 : a2;
  const double dlim = kill ? 0.0 : (st2 ? twice(from_bits(m)) : from_bits(m));
  const double hc = half(from_bits(ubits(dc) & kMag));  // |dcen|
  const unsigned long long r = ubits(dlim) < ubits(hc) ? ubits(dlim) : ubits(hc);
  const bool neg = (sbits(dc) < 0) && (ubits(hc) != 0ull);  // dcen < 0
  return from_bits(r | (neg ? kSign : 0ull));
}

}  // namespace f64x
}  // namespace e2d
