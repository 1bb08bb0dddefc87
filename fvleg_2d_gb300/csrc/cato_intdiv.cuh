// cato_intdiv.cuh -- IEEE-754 binary64 division and square root, rounded to nearest even, on the
// integer pipe.
//
// GB300 runs FP64 arithmetic at 1/64 of the FP32 rate, and a division or square root costs
// several FP64 instructions there.  The integer and FP32 pipes have room to spare.  These
// routines get the exact IEEE result from integer arithmetic on the significands:
//   1. an FP32 seed y0 ~ 1 / b (division) or 1 / sqrt(a) (square root) of the operand's
//      significand truncated to 24 bits, from the hardware approximation (any seed within 2^-21
//      relative will do);
//   2. one Newton-Raphson step of third order in 64-bit fixed point, y1 = y0 (1 + e + e^2) for
//      1/b with e = 1 - b y0, and y1 = y0 (1 + e/2 + 3e^2/8) for 1/sqrt(a) with e = 1 - a y0^2
//      (J.-M. Muller et al., Handbook of Floating-Point Arithmetic, 2nd ed., 2018, sections 4.7
//      and 11.3: Newton-Raphson iterations for the reciprocal and the reciprocal square root);
//   3. the quotient a y1 (or the root a y1) from three 32 x 32-bit partial products of the
//      64 x 64-bit product, within 43 units of 2^-61 (29 units of 2^-60 for the root) of the exact
//      value, far inside the 128 units the next step allows, then the nearest significand M1;
//   4. the exact rounding decision: the signs of the integer remainders
//      2^k A - (2 M1 +- 1) B (division) or 2^k A - (2 M1 +- 1)^2 (square root), computed
//      modulo 2^64 because their magnitudes are below 2^63, decide between M1 - 1, M1 and
//      M1 + 1, with ties to even.
// Exact scalings by 2^-1, 2^-2, 2^-3 and 2 (scale_down, scale_up1) are exponent steps here.
// Operands that are zero, subnormal, infinite or NaN, negative square-root operands and quotients
// outside the normal range take the hardware instruction instead (the caller's fallback).
// The same source compiles for the host, with correctly rounded seeds that a test hook moves by a
// few ulps; a host test compares the routines bit for bit with the hardware division and square
// root.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define CATO_HD __host__ __device__ __forceinline__
#else
#define CATO_HD static inline
#endif

namespace cato {
namespace intdiv {

CATO_HD uint64_t bits_of(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}
CATO_HD double double_of(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}
CATO_HD uint32_t fbits_of(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}
CATO_HD float float_of(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}
CATO_HD uint32_t umulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}
// floor(x y / 2^64) - d with 0 <= d < 3: the high half of a 64 x 64-bit product from three
// 32 x 32-bit products (the low x low product dropped, the cross products truncated)
CATO_HD uint64_t mulhi3(uint64_t x, uint64_t y) {
  const uint32_t xh = (uint32_t)(x >> 32), xl = (uint32_t)x, yh = (uint32_t)(y >> 32);
  const uint32_t yl = (uint32_t)y;
  return (uint64_t)xh * yh + (uint64_t)umulhi32(xh, yl) + (uint64_t)umulhi32(xl, yh);
}
// FP32 seeds y0 ~ 1/x and y0 ~ 1/sqrt(x) for x in [1, 4): on the device the single-instruction
// approximations (rcp.approx.ftz.f32, rsqrt.approx.ftz.f32).  The routines below are exact for
// any seed within 2^-21 relative of the true value (the error analysis keeps every fixed-point
// quantity inside 64 bits and the quotient within 4 units of its last bit); cato_gpu_check_divsqrt
// measures the hardware seeds' error over every input they get.  On the host the seeds are the
// correctly rounded values, moved by CATO_SEED_OFFSET units in the last place (a test hook that
// exercises seeds up to a few ulps off).
#if !defined(__CUDA_ARCH__) && defined(CATO_INTDIV_SEED_HOOK)
extern int seed_offset_ulps;
#define CATO_SEED_OFFSET seed_offset_ulps
#else
#define CATO_SEED_OFFSET 0
#endif
CATO_HD float recip_seed(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return float_of(fbits_of(1.0f / x) + (uint32_t)CATO_SEED_OFFSET);
#endif
}
CATO_HD float rsqrt_seed(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return float_of(fbits_of((float)(1.0 / __builtin_sqrt((double)x))) + (uint32_t)CATO_SEED_OFFSET);
#endif
}

constexpr uint64_t kFrac = 0x000fffffffffffffULL;
constexpr uint64_t kHid = 0x0010000000000000ULL;

// y * 2^30 as an integer for an FP32 seed y near [0.5, 1] (24 significant bits: exact)
CATO_HD uint32_t fixed30(float y) {
  const uint32_t yb = fbits_of(y);
  return ((yb & 0x7fffffu) | 0x800000u) << ((yb >> 23) - 120u);
}

// y0 (1 + t) * 2^62 for y0 = Y0 / 2^30 and t = T / 2^80 (floor of the correction term)
CATO_HD uint64_t refine62(uint32_t Y0, int64_t T) {
  const int64_t Th = T >> 32;                 // floor(T / 2^32)
  const uint64_t Tl = (uint32_t)T;
  const int64_t yt32 = (int64_t)Y0 * Th + (int64_t)(((uint64_t)Y0 * Tl) >> 32);  // floor(Y0 T / 2^32)
  return ((uint64_t)Y0 << 32) + (uint64_t)(yt32 >> 16);
}

// RN(a / b) as bits for normal a, b; ok = false when an operand is not normal or the quotient
// is not normal (the bits are then meaningless).
//
// With A, B the 53-bit significands (a = A 2^(ea-1075), b = B 2^(eb-1075)):
//   y0 ~ 1 / fb, fb = b' = B / 2^52 truncated to 24 bits, |1 - fb y0| <= 2^-21, so that
//   e = 1 - b' y0 has |e| < 1.25 2^-21 (the bounds below hold up to |e| = 2^-19);
//   E = 2^80 e = -(B Y0 / 4) mod 2^64 (Y0 is a multiple of 4), |E| < 2^61;
//   T = E + Eh^2 / 2^16 (Eh = floor(E / 2^32)) = 2^80 (e + e^2) within 2^-66;
//   Y1 = 2^62 y0 (1 + T / 2^80): |Y1 - 2^62 / b'| < 2 (the omitted e^3 term: 2^-57 at most);
//   H ~ A 2^11 Y1 / 2^64 (mulhi3): |H - 2^61 A / B| < 43;
//   n = 1 when H < 2^61 (quotient below 1), and with the quotient's significand in [1, 2) as
//   Hn = 2^n H, An = 2^n A: M1 = round(Hn / 2^9) is within 0.17 + 1/2 of X = 2^53 An / B, so
//   RN(X) is M1 - 1, M1 or M1 + 1, decided by the signs of Z = 2^53 An - (2 M1 + 1) B and
//   Z + 2 B (|Z| < 2^55).  Where n is taken wrongly (|H - 2^61| < 43), X lies within 0.17 of
//   2^52 or 2^53 and either choice rounds to the same value.
CATO_HD uint64_t div_bits(uint64_t ua, uint64_t ub, bool& ok) {
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
  const uint64_t A = (ua & kFrac) | kHid, B = (ub & kFrac) | kHid;
  const float fb = float_of(0x3f800000u | (uint32_t)((ub & kFrac) >> 29));
  const uint32_t Y0 = fixed30(recip_seed(fb));
  const int64_t E = (int64_t)(0ULL - B * (uint64_t)(Y0 >> 2));
  const int32_t Eh = (int32_t)(E >> 32);
  const int64_t T = E + (((int64_t)Eh * Eh) >> 16);
  const uint64_t Y1 = refine62(Y0, T);
  const uint64_t H = mulhi3(A << 11, Y1);
  const uint32_t n = (uint32_t)(H >> 61) ^ 1u;
  const uint64_t Hn = H << n, An = A << n;
  const uint64_t M1 = (Hn + 256u) >> 9;
  const int64_t Z = (int64_t)((An << 53) - (2 * M1 + 1) * B);
  uint64_t M = M1;
  if (Z > 0 || (Z == 0 && (M1 & 1))) {
    M = M1 + 1;
  } else {
    const int64_t W = Z + (int64_t)(2 * B);  // 2^53 An - (2 M1 - 1) B
    if (W < 0 || (W == 0 && (M1 & 1))) M = M1 - 1;
  }
  const int32_t Ef = (int32_t)ea - (int32_t)eb + 1023 - (int32_t)n;
  ok = (ea - 1u < 2046u) && (eb - 1u < 2046u) && (Ef >= 1) && (Ef <= 2045);
  const uint64_t sign = (ua ^ ub) & 0x8000000000000000ULL;
  // M in [2^52, 2^53]: M = 2^53 carries into the exponent field
  return sign | (((uint64_t)(uint32_t)Ef << 52) + (M - kHid));
}

// RN(sqrt(a)) as bits for normal a > 0; ok = false otherwise.
//
// a = A2 2^(2m) with A2 = A or 2A in [2^52, 2^54), a'' = A2 / 2^52 in [1, 4):
//   y0 ~ 1 / sqrt(fa), fa = a'' truncated to 24 bits, |1 - fa y0^2| <= 2^-21, so that
//   e = 1 - a'' y0^2 has |e| < 1.5 2^-21 (the bounds below hold up to |e| = 2^-19);
//   E = 2^80 e = -floor(A2 Y0^2 / 2^32) mod 2^64 (within 2 units), |E| < 2^61;
//   T = E / 2 + 3 floor(Eh^2 / 2^19) = 2^80 (e/2 + 3e^2/8);  Y1 = 2^62 y0 (1 + T / 2^80), within
//   6 units (the omitted 5e^3/16 term: 2^-58.7 at most);
//   H ~ A2 2^10 Y1 / 2^64 (mulhi3): |H - 2^60 sqrt(a'')| < 29, inside the 128 the rounding
//   allows;
//   M1 = round(H / 2^8), Z = 2^54 A2 - (2 M1 + 1)^2 (never 0), |Z| < 2^56.
CATO_HD uint64_t sqrt_bits(uint64_t ua, bool& ok) {
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu;
  const uint32_t odd = (ea & 1u) ^ 1u;  // the unbiased exponent ea - 1075 is odd
  const uint64_t A2 = ((ua & kFrac) | kHid) << odd;
  const float fa = float_of(((127u + odd) << 23) | (uint32_t)((ua & kFrac) >> 29));
  const uint32_t Y0 = fixed30(rsqrt_seed(fa));
  const uint64_t S = (uint64_t)Y0 * Y0;  // Y0^2 <= 2^60
  // floor(A2 S / 2^32) mod 2^64 from 32-bit halves (the carry out of the lowest product dropped)
  const uint32_t ah = (uint32_t)(A2 >> 32), al = (uint32_t)A2;
  const uint32_t sh = (uint32_t)(S >> 32), sl = (uint32_t)S;
  const uint64_t P = ((uint64_t)(ah * sh) << 32) + (uint64_t)ah * sl + (uint64_t)al * sh +
                     umulhi32(al, sl);
  const int64_t E = (int64_t)(0ULL - P);
  const int32_t Eh = (int32_t)(E >> 32);
  const int64_t T = (E >> 1) + 3 * (((int64_t)Eh * Eh) >> 19);
  const uint64_t Y1 = refine62(Y0, T);
  const uint64_t H = mulhi3(A2 << 10, Y1);
  const uint64_t M1 = (H + 128u) >> 8;
  const uint64_t N = 2 * M1 + 1;
  const int64_t Z = (int64_t)((A2 << 54) - N * N);
  uint64_t M = M1;
  if (Z > 0) M = M1 + 1;
  else if (Z + (int64_t)(8 * M1) < 0) M = M1 - 1;  // 2^54 A2 - (2 M1 - 1)^2 < 0
  ok = (ea - 1u < 2046u) && !(ua >> 63);
  const uint32_t Ef = 512u + ((ea - odd) >> 1);  // 1049 + (ea - 1075 - odd) / 2
  return (((uint64_t)Ef << 52) + (M - kHid));
}

// RN(a * b) as bits for normal a, b with a normal product; ok = false otherwise (zero, subnormal,
// infinite or NaN operands, products below the normal range or above the largest finite value;
// the bits are then meaningless).
//
// With A, B the 53-bit significands, the exact product P = A B (106 bits) is in [2^104, 2^106);
// t = 1 when P >= 2^105.  The rounded significand is M = floor(P / 2^(52+t)) plus one when the
// dropped bits exceed half a unit, or equal it with M odd (ties to even).  The dropped bits are
// left-aligned in a 64-bit word R, so that half a unit is 2^63.  M + 1 = 2^53 carries into the
// exponent field, and a carry out of the largest exponent gives the infinity that IEEE rounding
// to nearest gives.  Biased result exponent: ea + eb - 1023 + t.
CATO_HD uint64_t mul_bits(uint64_t ua, uint64_t ub, bool& ok) {
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
  const uint64_t A = (ua & kFrac) | kHid, B = (ub & kFrac) | kHid;
#ifdef __CUDA_ARCH__
  const uint64_t hi = __umul64hi(A, B), lo = A * B;
#else
  const unsigned __int128 P = (unsigned __int128)A * B;
  const uint64_t hi = (uint64_t)(P >> 64), lo = (uint64_t)P;
#endif
  const uint32_t t = (uint32_t)(hi >> 41);  // P >= 2^105
  const uint64_t M = (hi << (12u - t)) | (lo >> (52u + t));
  const uint64_t R = lo << (12u - t);
  const uint64_t up = (R > 0x8000000000000000ULL || (R == 0x8000000000000000ULL && (M & 1u)))
                          ? 1u : 0u;
  const int32_t E = (int32_t)(ea + eb + t) - 1023;
  ok = (ea - 1u < 2046u) && (eb - 1u < 2046u) && (E >= 1) && (E <= 2046);
  const uint64_t sign = (ua ^ ub) & 0x8000000000000000ULL;
  return sign | ((((uint64_t)(uint32_t)(E - 1)) << 52) + M + up);
}

// x * 2^-K (K = 1, 2, 3) and x * 2, equal to the IEEE products: an exponent step when the
// result is normal; below the normal range the significand is shifted with round-to-nearest-even;
// 2x overflows to infinity; infinities and NaN pass through.
template <int K> CATO_HD double scale_down(double x) {
  const uint64_t u = bits_of(x), a = u & 0x7fffffffffffffffULL;
  const uint32_t e = (uint32_t)(a >> 52);
  if (e > (uint32_t)K) return e == 0x7ffu ? x : double_of(u - ((uint64_t)K << 52));
  const uint64_t n = e == 0u ? a : (((a & kFrac) | kHid) << (e - 1u));  // |x| = n 2^-1074
  const uint64_t q = n >> K, rem = n & ((1ULL << K) - 1ULL), h = 1ULL << (K - 1);
  const uint64_t r = q + ((rem > h || (rem == h && (q & 1ULL))) ? 1ULL : 0ULL);
  return double_of((u & 0x8000000000000000ULL) | r);
}
CATO_HD double scale_up1(double x) {
  const uint64_t u = bits_of(x), a = u & 0x7fffffffffffffffULL, s = u & 0x8000000000000000ULL;
  const uint32_t e = (uint32_t)(a >> 52);
  if (e == 0u) return double_of(s | (a << 1));  // zero or subnormal: exact
  if (e >= 0x7feu) return e == 0x7ffu ? x : double_of(s | 0x7ff0000000000000ULL);
  return double_of(u + (1ULL << 52));
}

}  // namespace intdiv
}  // namespace cato
