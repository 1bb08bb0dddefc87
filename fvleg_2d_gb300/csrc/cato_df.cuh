// cato_df.cuh -- double-float ("df") arithmetic for the mixed_df path: a value is the unevaluated
// sum hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2, about 44 bits of precision computed
// entirely on the FP32 pipe (GB300 issues 64 FP32 operations per FP64 operation).
//
// The operations are the classical error-free transformations: Knuth's TwoSum, Dekker's
// FastTwoSum and the FMA-based TwoProduct, combined as in the double-double library of Hida, Li
// and Bailey ("Algorithms for quad-double precision floating point arithmetic", 2001) in their
// cheaper "sloppy" forms: the error of a sum is bounded relative to its operands (not its
// result), which keeps a difference of two nearby values as accurate as the values themselves.
// Division and square root take one correction step from an FP32 estimate.
//
// Every FP32 operation is written with an _rn intrinsic so that the compiler neither contracts
// nor reorders it, whatever the TU's --fmad setting.
#pragma once

#include <cuda_runtime.h>

namespace cato {

struct df {
  float hi, lo;
  df() = default;
  __host__ __device__ constexpr df(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr df(float f) : hi(f), lo(0.0f) {}
  __host__ __device__ constexpr df(int i) : hi((float)i), lo(0.0f) {}
  // Constants and host-side conversions (folded at compile time for literals).
  __host__ __device__ constexpr df(double d)
      : hi((float)d), lo((float)(d - (double)(float)d)) {}
};

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
  return df(s, e);
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ df operator-(df a) { return df(-a.hi, -a.lo); }

__device__ __forceinline__ df operator+(df a, df b) {
  const df s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }

__device__ __forceinline__ df operator*(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ df& operator+=(df& a, df b) { return a = a + b; }
__device__ __forceinline__ df& operator-=(df& a, df b) { return a = a - b; }
__device__ __forceinline__ df& operator*=(df& a, df b) { return a = a * b; }

// a / b: q1 = a.hi / b.hi, then q2 = (a - q1 b) / b.hi.  a.hi - q1*b.hi is exact (Sterbenz)
// because q1 is within a few ulp of the quotient.  Division by zero gives inf/NaN as FP32 does.
__device__ __forceinline__ df df_div(df a, df b) {
  const float q1 = __fdividef(a.hi, b.hi);
  if (!isfinite(q1)) return df(__fdiv_rn(a.hi, b.hi), 0.0f);
  const float p = __fmul_rn(q1, b.hi);
  float e = __fmaf_rn(q1, b.hi, -p);
  e = __fmaf_rn(q1, b.lo, e);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), e), a.lo);
  return fast_two_sum(q1, __fdividef(r, b.hi));
}

// sqrt(a): y = a.hi * rsqrt(a.hi), then y + (a - y^2) * rsqrt(a.hi) / 2.
__device__ __forceinline__ df df_sqrt(df a) {
  if (!(a.hi > 0.0f) || !isfinite(a.hi)) return df(sqrtf(a.hi), 0.0f);
  const float x = rsqrtf(a.hi);
  const float y = __fmul_rn(a.hi, x);
  const float p = __fmul_rn(y, y);
  const float e = __fmaf_rn(y, y, -p);
  const float d = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), e), a.lo);
  return fast_two_sum(y, __fmul_rn(__fmul_rn(d, x), 0.5f));
}

// ordering of normalised pairs: by hi, then lo (NaN compares false, as in IEEE)
__device__ __forceinline__ bool operator<(df a, df b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ bool operator>(df a, df b) { return b < a; }
__device__ __forceinline__ bool operator<=(df a, df b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo);
}
__device__ __forceinline__ bool operator>=(df a, df b) { return b <= a; }
__device__ __forceinline__ bool operator==(df a, df b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df a, df b) { return !(a == b); }

__device__ __forceinline__ df df_abs(df a) { return a.hi < 0.0f ? -a : a; }

}  // namespace cato
