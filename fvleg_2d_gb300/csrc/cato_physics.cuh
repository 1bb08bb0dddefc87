// cato_physics.cuh -- device arithmetic of CATO's hot path, templated on the compute type.
//
// R = double: the drop-in path.  Every expression keeps the reference's Fortran evaluation
// order (left-to-right, field-operator epsilon flushes, guarded divisions); the translation
// units that instantiate it are compiled with --fmad=false so each operation rounds on its own,
// which makes the results bit-identical to the CPU restatement of the reference.
// R = float: the mixed path's reconstruction and flux arithmetic (fast reciprocal division
// and square root); state accumulation stays FP64 in the stage kernel.
// R = df (cato_df.cuh): the mixed_df path, the same arithmetic in double-float pairs on the
// FP32 pipe (~44-bit precision); state accumulation stays FP64.
//
// Reference citations are file:line in smillerc/fvleg_2d.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "cato_df.cuh"
#include "cato_intdiv.cuh"

namespace cato {

// IEEE binary64 a / b and sqrt(a), rounded to nearest, for the FP64 path: the integer-pipe
// routines of cato_intdiv.cuh, and the hardware instruction for the operands they leave out
// (zero, subnormal, infinite or NaN operands, quotients outside the normal range).  The hardware
// forms are kept out of line so that the compiler branches to them instead of evaluating them
// alongside.  div_rn and sqrt_rn are out of line too: one copy of each (~80 instructions) per
// kernel instead of one per call site keeps the stage kernels inside the instruction cache
// (+18 % FP64 cell-updates/s on the 4096^2 quadrant, +55 % on the serving mix, where five flux
// kernels run side by side).
static __device__ __noinline__ double div_hw(double a, double b) { return a / b; }
static __device__ __noinline__ double sqrt_hw(double a) { return ::sqrt(a); }
static __device__ __noinline__ double div_rn(double a, double b) {
  bool ok;
  const uint64_t q = intdiv::div_bits(intdiv::bits_of(a), intdiv::bits_of(b), ok);
  return ok ? intdiv::double_of(q) : div_hw(a, b);
}
static __device__ __noinline__ double sqrt_rn(double a) {
  bool ok;
  const uint64_t r = intdiv::sqrt_bits(intdiv::bits_of(a), ok);
  return ok ? intdiv::double_of(r) : sqrt_hw(a);
}
// IEEE binary64 a * b on the integer pipe (intdiv::mul_bits), bit-identical to the FP64
// instruction: a zero operand times a finite one is the zero with the product's sign; operands
// or products outside the normal range take the hardware instruction.  Out of line, as div_rn.
static __device__ __noinline__ double mul_hw(double a, double b) { return a * b; }
static __device__ __noinline__ double mul_rn(double a, double b) {
  const uint64_t ua = intdiv::bits_of(a), ub = intdiv::bits_of(b);
  const uint64_t za = ua << 1, zb = ub << 1;
  if ((za == 0ULL || zb == 0ULL) && za < 0xffe0000000000000ULL && zb < 0xffe0000000000000ULL)
    return intdiv::double_of((ua ^ ub) & 0x8000000000000000ULL);
  bool ok;
  const uint64_t r = intdiv::mul_bits(ua, ub, ok);
  return ok ? intdiv::double_of(r) : mul_hw(a, b);
}

enum { FLUX_AUSMPW = 0, FLUX_SLAU = 1, FLUX_SLAU2 = 2, FLUX_SD_SLAU = 3, FLUX_SD_SLAU2 = 4,
       FLUX_ROE = 5, FLUX_AUSM_UP = 6, FLUX_HLLC = 7, FLUX_M_AUSMPW = 8 };
enum { LIM_MINMOD = 0, LIM_SUPERBEE = 1, LIM_VANLEER = 2, LIM_MLP3 = 3, LIM_MLP5 = 4 };
enum { BC_ZERO_GRADIENT = 0, BC_SYMMETRY = 1, BC_PERIODIC = 2, BC_OUTLET = 3,
       BC_PRESSURE_INPUT = 4, BC_EXCHANGE = 5 };
enum { SIDE_PX = 0, SIDE_PY = 1, SIDE_MX = 2, SIDE_MY = 3 };

// Status word bits written by the kernels (mapped to the reference's error codes on the host).
enum { ST_NEG_DENSITY = 1, ST_NEG_PRESSURE = 2, ST_NAN = 4,
       ST_BC_INPUT = 8 /* pressure-input target below tiny (the reference stops) */ };

template <typename R> struct Num;
// the mixed path's FP32 compute type (its arithmetic skips the reference's FP64-scale epsilon
// flushes, which cannot fire at FP32 resolution for data of normal magnitude)
template <typename R> constexpr bool kFP32 = false;
template <> constexpr bool kFP32<float> = true;

template <> struct Num<double> {
  static constexpr double eps = 2.220446049250313080847263336181640625e-16;  // epsilon(1.0_rk)
  static constexpr double tiny = 2.2250738585072013830902327173324040642e-308; // tiny(1.0_rk)
  // IEEE a / b on the integer pipe (div_rn).  A signed zero over a finite non-zero b (flat
  // data) is the zero with the sign of the product, decided before the general routine.
  static __device__ __forceinline__ double div(double a, double b) {
    const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
    const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
    if ((ua << 1) == 0ULL && (ub << 1) != 0ULL && ((ub >> 52) & 0x7ffULL) != 0x7ffULL)
      return __longlong_as_double((long long)((ua ^ ub) & 0x8000000000000000ULL));
    return div_rn(a, b);
  }
  // sqrt(+-0) = +-0 (a zero velocity), else sqrt_rn
  static __device__ __forceinline__ double sqrt(double a) {
    if (((unsigned long long)__double_as_longlong(a) << 1) == 0ULL) return a;
    return sqrt_rn(a);
  }
  // a * b on the integer pipe (mul_rn)
  static __device__ __forceinline__ double mul(double a, double b) { return mul_rn(a, b); }
};

template <> struct Num<float> {
  static constexpr float eps = 2.220446049250313080847263336181640625e-16f;
  static constexpr float tiny = FLT_MIN;
  static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
  static __device__ __forceinline__ float sqrt(float a) { return ::sqrtf(a); }
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
};

template <> struct Num<df> {
  static constexpr df eps = df(2.220446049250313080847263336181640625e-16f, 0.0f);
  static constexpr df tiny = df(FLT_MIN, 0.0f);
  static __device__ __forceinline__ df div(df a, df b) { return df_div(a, b); }
  static __device__ __forceinline__ df sqrt(df a) { return df_sqrt(a); }
  static __device__ __forceinline__ df mul(df a, df b) { return a * b; }
};

// FP64: the reference's MAX/MIN as compare-and-select (identical signed-zero behaviour to the
// CPU restatement).  FP32 (mixed path): single-instruction min/max.
template <typename R> __device__ __forceinline__ R rmax(R a, R b) { return (a < b) ? b : a; }
template <typename R> __device__ __forceinline__ R rmin(R a, R b) { return (b < a) ? b : a; }
template <> __device__ __forceinline__ float rmax<float>(float a, float b) { return fmaxf(a, b); }
// FP64 compare-and-select on the integer pipe: the sign-magnitude bits map to a monotone signed
// key (+0 and -0 share key 0); a NaN operand makes the comparison false, as in IEEE.
__device__ __forceinline__ bool d_isnan(double x) {
  return ((unsigned long long)__double_as_longlong(x) << 1) > 0xffe0000000000000ULL;
}
__device__ __forceinline__ long long d_key(double x) {
  const long long b = __double_as_longlong(x);
  return b >= 0 ? b : -(b & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool d_less(double a, double b) {
  return d_key(a) < d_key(b) && !d_isnan(a) && !d_isnan(b);
}
template <> __device__ __forceinline__ double rmax<double>(double a, double b) {
  return d_less(a, b) ? b : a;
}
template <> __device__ __forceinline__ double rmin<double>(double a, double b) {
  return d_less(b, a) ? b : a;
}
// x <= 0 (false for NaN)
template <typename R> __device__ __forceinline__ bool nonpos(R x) { return x <= R(0); }
template <> __device__ __forceinline__ bool nonpos<double>(double x) {
  const long long b = __double_as_longlong(x);
  return (b < 0 || (b << 1) == 0) && !d_isnan(x);
}
// a <= b, x >= 0, x > 0, x < 0 (IEEE: false with a NaN operand); FP64 on the integer pipe
template <typename R> __device__ __forceinline__ bool le(R a, R b) { return a <= b; }
template <typename R> __device__ __forceinline__ bool ge0(R x) { return x >= R(0); }
template <typename R> __device__ __forceinline__ bool gt0(R x) { return x > R(0); }
template <typename R> __device__ __forceinline__ bool lt0(R x) { return x < R(0); }
template <> __device__ __forceinline__ bool le<double>(double a, double b) {
  return d_key(a) <= d_key(b) && !d_isnan(a) && !d_isnan(b);
}
template <> __device__ __forceinline__ bool ge0<double>(double x) {
  const long long b = __double_as_longlong(x);
  return (b >= 0 || (b << 1) == 0) && !d_isnan(x);
}
template <> __device__ __forceinline__ bool gt0<double>(double x) {
  const long long b = __double_as_longlong(x);
  return b > 0 && !d_isnan(x);
}
template <> __device__ __forceinline__ bool lt0<double>(double x) {
  const long long b = __double_as_longlong(x);
  return b < 0 && (b << 1) != 0 && !d_isnan(x);
}
template <> __device__ __forceinline__ float rmin<float>(float a, float b) { return fminf(a, b); }
template <typename R> __device__ __forceinline__ R rabs(R a) { return fabs(a); }
template <> __device__ __forceinline__ df rabs<df>(df a) { return df_abs(a); }
// Fortran SIGN(1.0, x)
template <typename R> __device__ __forceinline__ R fsign1(R x) { return signbit(x) ? R(-1) : R(1); }
template <> __device__ __forceinline__ df fsign1<df>(df x) {
  return signbit(x.hi) ? df(-1.0f) : df(1.0f);
}

// R(0.5) * x, R(0.25) * x, R(0.125) * x, R(2) * x
template <typename R> __device__ __forceinline__ R half(R x) { return R(0.5) * x; }
template <typename R> __device__ __forceinline__ R quarter(R x) { return R(0.25) * x; }
template <typename R> __device__ __forceinline__ R eighth(R x) { return R(0.125) * x; }
template <typename R> __device__ __forceinline__ R twice(R x) { return R(2) * x; }
// FP64: exact scalings on the integer pipe (intdiv::scale_down / scale_up1)
template <> __device__ __forceinline__ double half<double>(double x) {
  return intdiv::scale_down<1>(x);
}
template <> __device__ __forceinline__ double quarter<double>(double x) {
  return intdiv::scale_down<2>(x);
}
template <> __device__ __forceinline__ double eighth<double>(double x) {
  return intdiv::scale_down<3>(x);
}
template <> __device__ __forceinline__ double twice<double>(double x) { return intdiv::scale_up1(x); }

// a + b * R(0): the reference's products with the zero component of an axis-aligned unit normal.
// FP64 on the integer pipe: b * 0 is the zero with the sign of b when b is finite (NaN
// otherwise), and a + (+-0) is a unless a is a zero, where -0 results only from -0 + -0.
template <typename R> __device__ __forceinline__ R add_mul0(R a, R b) { return a + b * R(0); }
template <> __device__ __forceinline__ double add_mul0<double>(double a, double b) {
  const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
  const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
  if ((ub << 1) >= 0xffe0000000000000ULL) return a + b * 0.0;  // b infinite or NaN
  if ((ua << 1) != 0ULL) return a;
  return ((ua & ub) >> 63) ? -0.0 : 0.0;
}

// |x| < c for c > 0 without an FP compare: bit patterns of non-negative IEEE values order like
// unsigned integers and NaN compares false, as the reference's ABS(x) < c does.
__device__ __forceinline__ bool abs_lt(double x, double c) {
  unsigned long long bx = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
  return bx < (unsigned long long)__double_as_longlong(c);
}
__device__ __forceinline__ bool abs_lt(float x, float c) { return fabsf(x) < c; }
__device__ __forceinline__ bool abs_lt(df x, df c) { return df_abs(x) < c; }

// abs_lt(x / cs, 1e-13) with x / cs rounded, as the Mach filter of calculate_derived_quantities
// (mod_fluid.f90:579-588; x below tiny counts as a zero Mach number).  The quotient is only
// formed when the exponents leave the answer open: for normal x and cs with biased exponents
// Ex, Ec, |x / cs| lies in (2^(Ex-Ec-1), 2^(Ex-Ec+1)), and 1e-13 lies in [2^-44, 2^-43), so
// Ex - Ec >= -42 puts the rounded quotient at or above 2^-43 (not below 1e-13) and Ex - Ec <= -46
// puts it at or below 2^-45 (below).  The division runs on the FP64 pipe, the test on the
// integer pipe.
__device__ __forceinline__ bool mach_below_1e13(double x, double cs) {
  if (abs_lt(x, Num<double>::tiny)) return true;
  const int ex = (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffULL);
  const int ec = (int)(((unsigned long long)__double_as_longlong(cs) >> 52) & 0x7ffULL);
  if (ex >= 1 && ex <= 2046 && ec >= 1 && ec <= 2046) {
    if (ex - ec >= -42) return false;
    if (ex - ec <= -46) return true;
  }
  return abs_lt(div_rn(x, cs), 1e-13);
}

// FP64 <-> FP32 conversion on the integer pipe (GB300's F2F shares the narrow FP64 pipe).
// d2f: round-to-nearest-even, values below FLT_MIN flush to signed zero, NaN stays NaN.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float d2f_int(double d) {
  unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  unsigned sign = hi & 0x80000000u;
  int e = (int)((hi >> 20) & 0x7ffu);
  unsigned mf = ((hi & 0xfffffu) << 3) | (lo >> 29);
  unsigned rem = lo & 0x1fffffffu;
  int fe = e - 896;
  unsigned res = sign | ((unsigned)fe << 23) | mf;
  res += (rem > 0x10000000u || (rem == 0x10000000u && (mf & 1u))) ? 1u : 0u;
  if (fe <= 0) res = sign;
  if (fe >= 255) res = sign | 0x7f800000u;
  if (e == 0x7ff && (((hi & 0xfffffu) | lo) != 0u)) res = 0x7fc00000u;
  return __uint_as_float(res);
}
// f2d: exact; float denormals flush to zero.
__device__ __forceinline__ double f2d_int(float f) {
  unsigned b = __float_as_uint(f);
  unsigned sign = b & 0x80000000u, e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  unsigned hi, lo = m << 29;
  if (e == 0u) { hi = sign; lo = 0u; }
  else if (e == 255u) hi = sign | 0x7ff00000u | (m >> 3);
  else hi = sign | ((e + 896u) << 20) | (m >> 3);
  return __hiloint2double((int)hi, (int)lo);
}

// FP64 -> FP32 for the mixed path's stencil values: the exponent rebiased and the fraction
// truncated to 23 bits (at most one FP32 unit in the last place towards zero from the rounded
// value); magnitudes below FLT_MIN become a signed zero.  One funnel shift, an add, a select and
// two logic operations, against ~14 integer operations for the rounded d2f_int.  Valid for
// finite magnitudes below 2^128 (conserved states); NaN and infinity are not preserved, so the
// state checks keep d2f_int.
__device__ __forceinline__ float d2f_fast(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  // bits 31..23: the low 9 bits of the FP64 exponent, minus 384 = the FP32 exponent (mod 512)
  const unsigned m = __funnelshift_l(lo, hi, 3) - (384u << 23);
  const unsigned sign = hi & 0x80000000u;
  return __uint_as_float((hi << 1) >= (897u << 21) ? (m | sign) : sign);
}

// FP64 <-> df: hi = the FP64 value rounded to FP32, lo = the (exact) remainder rounded to FP32;
// one FP64 add, the conversions on the integer pipe.
__device__ __forceinline__ df to_df(double d) {
  const float h = d2f_int(d);
  return df(h, d2f_int(d - f2d_int(h)));
}
__device__ __forceinline__ double from_df(df a) { return f2d_int(a.hi) + f2d_int(a.lo); }

// ---------------------------------------------------------------------------------------------
// Primitive recovery
// ---------------------------------------------------------------------------------------------
// FP64: eos%conserved_to_primitive through the field operators (equation_of_state.f90:297-314;
// field_2d_cpu_operators.f90:84-420: '+'/'-' flush |x|<eps to 0, field/field returns 0 when
// |lhs|<tiny), eos%sound_speed (:269-278) and the Mach filter of calculate_derived_quantities
// (mod_fluid.f90:564-591).
__device__ __forceinline__ void prim_from_cons(double g, double g1, double r, double ru,
                                               double rv, double rE, double& u, double& v,
                                               double& p, double& cs) {
  const double EPS = Num<double>::eps, TINY = Num<double>::tiny;
  u = abs_lt(ru, TINY) ? 0.0 : div_rn(ru, r);
  v = abs_lt(rv, TINY) ? 0.0 : div_rn(rv, r);
  double e = abs_lt(rE, TINY) ? 0.0 : div_rn(rE, r);
  // explicitly rounded: identical in translation units built with FMA contraction
  double s = __dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v));
  if (abs_lt(s, EPS)) s = 0.0;
  double h = half(s);
  double dd = e - h;
  if (abs_lt(dd, EPS)) dd = 0.0;
  p = (r * g1) * dd;
  double pr = abs_lt(p, TINY) ? 0.0 : div_rn(p, r);
  cs = Num<double>::sqrt(pr * g);
  // mach_u = u / cs, mach_v = v / cs, then |mach| < 1e-13 zeroes the velocity
  if (mach_below_1e13(u, cs)) u = 0.0;  // each test reads only its own component and cs
  if (mach_below_1e13(v, cs)) v = 0.0;
}

// The FP64 recovery out of line, for the double-float path's rare cells where its own
// arithmetic cannot resolve the pressure (see near_vacuum)
static __device__ __noinline__ void prim_from_cons_f64(double g, double r, double ru, double rv,
                                                       double rE, double& u, double& v,
                                                       double& p) {
  double cs;
  prim_from_cons(g, __dsub_rn(g, 1.0), r, ru, rv, rE, u, v, p, cs);
}

// Whether the double-float pressure p, recovered as (gamma - 1)(rho E - kinetic energy), is too
// close to zero for its arithmetic: the difference loses all the digits a cancellation of
// rho E against the kinetic energy takes, and the FP64 recovery flushes a specific internal
// energy below epsilon to an exact zero pressure (field_2d_cpu_operators.f90 '-' flush).  Such
// cells (near-vacuum expansions) take the FP64 recovery from the FP64 conserved state, so that
// their pressure, its zero and its sign (the negative-pressure check) are the FP64 path's.
// rel: where p loses its digits (double-float: below ~1e-4 of rho E, with margin).
__device__ __forceinline__ bool near_vacuum(float p, float rE, float rel) {
  return !(fabsf(p) >= rel * fabsf(rE));
}

// FP32 (mixed path): same quantities with one reciprocal of rho; Mach filter as |u| < 1e-13 cs.
__device__ __forceinline__ void prim_from_cons(float g, float g1, float r, float ru, float rv,
                                               float rE, float& u, float& v, float& p, float& cs) {
  float ir = __fdividef(1.0f, r);
  u = ru * ir;
  v = rv * ir;
  p = g1 * (rE - 0.5f * r * (u * u + v * v));
  cs = sqrtf(g * p * ir);
  if (fabsf(v) < 1e-13f * cs) v = 0.0f;
  if (fabsf(u) < 1e-13f * cs) u = 0.0f;
}

// df (mixed_df path): as the FP32 variant, in double-float; the Mach filter compares against an
// FP32 sound speed (it only decides whether a velocity below 1e-13 c is set to zero).
__device__ __forceinline__ void prim_from_cons(df g, df g1, df r, df ru, df rv, df rE, df& u,
                                               df& v, df& p, df& cs, bool want_cs) {
  const df ir = df_div(df(1.0f), r);
  u = ru * ir;
  v = rv * ir;
  p = g1 * (rE - df(0.5f) * r * (u * u + v * v));
  const float csf = sqrtf(fmaxf(g.hi * p.hi * ir.hi, 0.0f));
  if (want_cs) cs = df_sqrt(g * p * ir);
  if (fabsf(v.hi) < 1e-13f * csf) v = df(0.0f);
  if (fabsf(u.hi) < 1e-13f * csf) u = df(0.0f);
}

// ---------------------------------------------------------------------------------------------
// Reconstruction: MUSCL TVD2 (muscl_tvd2.fypp:172-223) and MLP3/MLP5 (muscl_mlp.fypp:190-281).
// Stencil values along the edge normal: qm2..qp3 = cells i-2 .. i+3 (edge between i and i+1);
// transverse for MLP: t0p/t0m = cell i at tangential +-1, t1p/t1m = cell i+1 at +-1.
// ---------------------------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R tvd_phi(int lim, R r) {
  if (lim == LIM_MINMOD) return rmax(R(0), rmin(r, R(1)));
  if (lim == LIM_SUPERBEE) return rmax(rmax(R(0), rmin(twice(r), R(1))), rmin(r, R(2)));
  // "vanleer" (muscl_tvd2.fypp:199-200); for r <= 0 the numerator r + |r| is +0 and so is
  // the quotient (1 + |r| >= 1): skip the division
  if (nonpos(r)) return R(0);
  return Num<R>::div(twice(r), R(1) + r);  // r > 0: r + |r| = 2r exactly, |r| = r
}

// phi(num / den).  Every limiter gives +0 for r < 0, and FP64 knows r < 0 without dividing when
// num and den are finite, non-zero and of opposite signs (the quotient is then negative, -inf or
// -0); the sign test runs on the integer pipe.
template <typename R>
__device__ __forceinline__ R tvd_phi_of(int lim, R num, R den) {
  if constexpr (std::is_same<R, double>::value) {
    const long long bn = __double_as_longlong(num), bd = __double_as_longlong(den);
    const unsigned long long an = (unsigned long long)bn << 1, ad = (unsigned long long)bd << 1;
    // non-zero (an, ad != 0), finite (exponent != 0x7ff: shifted < 0xffe0...), signs differ
    if (an != 0ULL && ad != 0ULL && an < 0xffe0000000000000ULL && ad < 0xffe0000000000000ULL &&
        ((bn ^ bd) < 0))
      return R(0);
  }
  return tvd_phi(lim, Num<R>::div(num, den));
}

// q + (0.5 phi) d, or q - (0.5 phi) d (minus).  FP64: 0.5 phi is an exponent step, and phi = +0
// (flat data, or a limiter at zero) gives the product +-0 with the sign of d (d finite), so the
// sum is q itself unless q is a signed zero, where IEEE gives -0 only for -0 + -0.
template <typename R>
__device__ __forceinline__ R slope_step(R q, R phi, R d, bool minus) {
  return minus ? q - R(0.5) * phi * d : q + R(0.5) * phi * d;
}
template <>
__device__ __forceinline__ double slope_step<double>(double q, double phi, double d, bool minus) {
  const unsigned long long bq = (unsigned long long)__double_as_longlong(q);
  const unsigned long long bd = (unsigned long long)__double_as_longlong(d);
  if (__double_as_longlong(phi) == 0LL && ((bd << 1) < 0xffe0000000000000ULL)) {
    if ((bq << 1) != 0ULL) return q;
    const bool zneg = ((bd >> 63) != 0ULL) != minus;  // the sign of the zero added to q
    return ((bq >> 63) && zneg) ? -0.0 : 0.0;
  }
  const double t = half(phi) * d;
  return minus ? q - t : q + t;
}

// phi(d0 / (dq + 1e-16)).  FP64: d0 = +-0 over a finite dq gives r = +-0 (the denominator is
// finite and non-zero: |dq| is 0 or at least epsilon after the flush) and phi(+-0) = +0 for
// every limiter, without the regularising addition.
template <typename R>
__device__ __forceinline__ R tvd_phi_edge(int lim, R d0, R dq) {
  return tvd_phi_of(lim, d0, dq + R(1e-16));
}
template <>
__device__ __forceinline__ double tvd_phi_edge<double>(int lim, double d0, double dq) {
  const unsigned long long b0 = (unsigned long long)__double_as_longlong(d0);
  const unsigned long long bq = (unsigned long long)__double_as_longlong(dq);
  if ((b0 << 1) == 0ULL && (bq << 1) < 0xffe0000000000000ULL) return 0.0;
  return tvd_phi_of(lim, d0, dq + 1e-16);
}

template <typename R>
__device__ __forceinline__ void recon_tvd2(int lim, R qm1, R q0, R qp1, R qp2, R& L, R& Rr) {
  const R EPS = Num<R>::eps;
  R dm = q0 - qm1, d0 = qp1 - q0, dp = qp2 - qp1;
  if constexpr (!kFP32<R>) {  // FP32 differences below 2.2e-16 need |q| < 1e-9: no flush
    if (abs_lt(dm, EPS)) dm = R(0);
    if (abs_lt(d0, EPS)) d0 = R(0);
    if (abs_lt(dp, EPS)) dp = R(0);
  }
  L = slope_step(q0, tvd_phi_edge(lim, d0, dm), dm, false);
  Rr = slope_step(qp1, tvd_phi_edge(lim, d0, dp), dp, true);
}

// FP64 TVD2 edge values out of line: one copy per kernel instead of one per variable and
// direction keeps the stage kernel inside the instruction cache
struct EdgePair {
  double L, R;
};
static __device__ __noinline__ EdgePair recon_tvd2_f64(int lim, double qm1, double q0, double qp1,
                                                      double qp2) {
  EdgePair e;
  recon_tvd2<double>(lim, qm1, q0, qp1, qp2, e.L, e.R);
  return e;
}

// FP32 (mixed path): the limited slope phi(r) * dq without the ratio.  For r = d0/dq > 0,
// minmod gives min(r, 1) dq = (|d0| < |dq| ? d0 : dq), superbee picks one of 2 d0, dq, d0, 2 dq,
// and van Leer's 2r/(1+r) dq = 2 d0 dq / (dq + d0); r <= 0 gives 0.  Written with selects (no
// data-dependent branches: the warp stays converged); the limiter id is uniform.
__device__ __forceinline__ float tvd_slope_f32(int lim, float d0, float dq) {
  const bool pos = d0 * dq > 0.0f;
  const float a0 = fabsf(d0), aq = fabsf(dq);
  float s;
  if (lim == LIM_MINMOD) {
    s = a0 < aq ? d0 : dq;
  } else if (lim == LIM_SUPERBEE) {
    const float lo = (2.0f * a0 <= aq) ? 2.0f * d0 : dq;   // r <= 1
    const float hi = (a0 <= 2.0f * aq) ? d0 : 2.0f * dq;   // r > 1
    s = (a0 <= aq) ? lo : hi;
  } else {
    s = __fdividef(2.0f * d0 * dq, dq + d0);
  }
  return pos ? s : 0.0f;
}

template <>
__device__ __forceinline__ void recon_tvd2<float>(int lim, float qm1, float q0, float qp1,
                                                  float qp2, float& L, float& Rr) {
  const float dm = q0 - qm1, d0 = qp1 - q0, dp = qp2 - qp1;
  L = q0 + 0.5f * tvd_slope_f32(lim, d0, dm);
  Rr = qp1 - 0.5f * tvd_slope_f32(lim, d0, dp);
}

// num / den is certainly <= 0 and not NaN: num = +-0 over a finite non-zero den, or finite
// non-zero operands of opposite signs (integer pipe)
__device__ __forceinline__ bool ratio_nonpos(double num, double den) {
  const long long bn = __double_as_longlong(num), bd = __double_as_longlong(den);
  const unsigned long long an = (unsigned long long)bn << 1, ad = (unsigned long long)bd << 1;
  if (ad == 0ULL || ad >= 0xffe0000000000000ULL) return false;  // den zero, inf or NaN
  if (an == 0ULL) return true;
  return an < 0xffe0000000000000ULL && ((bn ^ bd) < 0);
}

template <typename R, int ORDER>
__device__ __forceinline__ void recon_mlp(R qm2, R qm1, R q0, R qp1, R qp2, R qp3, R t0p, R t0m,
                                          R t1p, R t1m, R& L, R& Rr) {
  const R EPS = Num<R>::eps;
  const R S = R(1e-30);  // SMALL_NUM, muscl_mlp.fypp:122
  R dm = q0 - qm1, d0 = qp1 - q0, dp = qp2 - qp1;
  if constexpr (!kFP32<R>) {
    if (abs_lt(dm, EPS)) dm = R(0);
    if (abs_lt(d0, EPS)) d0 = R(0);
    if (abs_lt(dp, EPS)) dp = R(0);
  }
  // FP64: a side whose ratio is <= 0 has a limited slope of +0 whatever beta and alpha are
  // (alpha is clamped to [1, 2], so min(alpha r, alpha, beta) <= 0 and max(0, .) = +0); its
  // beta and alpha, which take most of the divisions, are skipped
  bool zL = false, zR = false;
  if constexpr (std::is_same<R, double>::value) {
    zL = ratio_nonpos(d0, dm + S);
    zR = ratio_nonpos(d0, dp + S);
  }
  R phiL = R(0), phiR = R(0);
  if (!zL || !zR) {
    R rR_p1 = Num<R>::div(d0, dp + S);
    R rL = Num<R>::div(d0, dm + S);
    R bL = R(0), bR = R(0);
    if (ORDER == 5) {
      R dm3 = qm1 - qm2, dp5 = qp3 - qp2;
      if constexpr (!kFP32<R>) {
        if (abs_lt(dm3, EPS)) dm3 = R(0);
        if (abs_lt(dp5, EPS)) dp5 = R(0);
      }
      if (!zL) {
        R rL_m1 = Num<R>::div(dm, dm3 + S);
        R rL_p1 = Num<R>::div(dp, d0 + S);
        bL = Num<R>::div(
            (((Num<R>::div(R(-2), rL_m1 + S)) + R(11)) + R(24) * rL) - R(3) * rL * rL_p1, R(30));
      }
      if (!zR) {
        R rR_p2 = Num<R>::div(dp, dp5 + S);
        R rR = Num<R>::div(dm, d0 + S);
        bR = Num<R>::div((((Num<R>::div(R(-2), rR_p2 + S)) + R(11)) + R(24) * rR_p1) -
                             R(3) * rR_p1 * rR,
                         R(30));
      }
    } else {
      if (!zL) bL = Num<R>::div(R(1) + twice(rL), R(3));
      if (!zR) bR = Num<R>::div(R(1) + twice(rR_p1), R(3));
    }
    R tt = Num<R>::div(rabs(t0p - t0m), rabs(qp1 - qm1) + S);
    R tt1 = Num<R>::div(rabs(t1p - t1m), rabs(qp2 - q0) + S);
    if (!zL) {
      R aLt = Num<R>::div(twice(rmax(R(1), rL)) * (R(1) + rmax(R(0), Num<R>::div(tt1, rR_p1 + S))),
                          R(1) + tt);
      R aL = rmax(R(1), rmin(R(2), aLt));
      phiL = rmax(R(0), rmin(rmin(aL * rL, aL), bL));
    }
    if (!zR) {
      R aRt = Num<R>::div(twice(rmax(R(1), rR_p1)) * (R(1) + rmax(R(0), Num<R>::div(tt, rL + S))),
                          R(1) + tt1);
      R aR = rmax(R(1), rmin(R(2), aRt));
      phiR = rmax(R(0), rmin(rmin(aR * rR_p1, aR), bR));
    }
  }
  L = slope_step(q0, phiL, dm, false);
  Rr = slope_step(qp1, phiR, dp, true);
}

// FP64 MLP edge values out of line (one copy per kernel, as recon_tvd2_f64)
template <int ORDER>
static __device__ __noinline__ EdgePair recon_mlp_f64(double qm2, double qm1, double q0, double qp1,
                                                     double qp2, double qp3, double t0p,
                                                     double t0m, double t1p, double t1m) {
  EdgePair e;
  recon_mlp<double, ORDER>(qm2, qm1, q0, qp1, qp2, qp3, t0p, t0m, t1p, t1m, e.L, e.R);
  return e;
}

// ---------------------------------------------------------------------------------------------
// Double-float reconstruction (mixed_df).  The limited slope phi(r) * dq is, for each branch of
// the limiter, an algebraic combination of the slope differences themselves: with r = d0/dm,
// r * dm = d0, (1 + 2r)/3 * dm = (dm + 2 d0)/3, and the MLP5 coefficient times dm is the
// fifth-order combination (-2 dm3 + 11 dm + 24 d0 - 3 dp)/30.  So the slope candidates are formed
// in double-float from the double-float differences without the ratio divisions, and every
// choice between them is a comparison of those double-float candidates (exact for normalised
// pairs), so a near-tie never picks a branch on FP32 rounding.  Only the MLP alpha, which needs
// divisions, is estimated in FP32 first and formed in double-float when the estimate cannot
// settle the choice.  The reference's 1e-16 / 1e-30 regularisations only matter for differences
// at the epsilon flush threshold, where the slope term is itself ~1e-16.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ df df_half(df a) { return df(a.hi * 0.5f, a.lo * 0.5f); }  // exact
__device__ __forceinline__ df df_twice(df a) { return df(a.hi * 2.0f, a.lo * 2.0f); }  // exact
__device__ __forceinline__ df df_scale(df a, float c) { return a * df(c); }

// r = d0 / dq <= 0 from the signs of normalised pairs (exact): a zero, or opposite signs
__device__ __forceinline__ bool df_ratio_nonpos(df D0, df Dq) {
  return D0.hi == 0.0f || Dq.hi == 0.0f || ((D0.hi > 0.0f) != (Dq.hi > 0.0f));
}

// TVD2 slope phi(r) * dq for r = d0 / dq (dq = dm for the left state, dp for the right)
__device__ __forceinline__ df tvd_slope_df(int lim, df D0, df Dq) {
  if (df_ratio_nonpos(D0, Dq)) return df(0.0f);  // r <= 0
  const df a0 = df_abs(D0), aq = df_abs(Dq);    // r = a0 / aq > 0
  if (lim == LIM_MINMOD) return a0 < aq ? D0 : Dq;            // min(r, 1) * dq
  if (lim == LIM_SUPERBEE) {                                    // max(min(2r, 1), min(r, 2)) * dq
    if (df_twice(a0) <= aq) return df_twice(D0);
    if (a0 <= aq) return Dq;
    if (a0 <= df_twice(aq)) return D0;
    return df_twice(Dq);
  }
  // van Leer: 2r / (1 + r) * dq = 2 d0 dq / (dq + d0)
  return df_div(df_twice(D0 * Dq), Dq + D0);
}

__device__ __forceinline__ df flushed(df d) {
  return fabsf(d.hi) < 2.220446049250313080847263336181640625e-16f ? df(0.0f) : d;
}

// Double-float edge values out of line (one copy per kernel instead of one per variable and
// direction: the double-float stage kernels otherwise outgrow the instruction cache)
struct DfPair {
  df L, R;
};
static __device__ __noinline__ DfPair recon_tvd2_df(int lim, df qm1, df q0, df qp1, df qp2) {
  const df Dm = flushed(q0 - qm1), D0 = flushed(qp1 - q0), Dp = flushed(qp2 - qp1);
  DfPair e;
  e.L = q0 + df_half(tvd_slope_df(lim, D0, Dm));
  e.R = qp1 - df_half(tvd_slope_df(lim, D0, Dp));
  return e;
}

template <>
__device__ __forceinline__ void recon_tvd2<df>(int lim, df qm1, df q0, df qp1, df qp2, df& L,
                                               df& Rr) {
  const DfPair e = recon_tvd2_df(lim, qm1, q0, qp1, qp2);
  L = e.L;
  Rr = e.R;
}

// One side of the MLP limiter: the slope phi * dq, phi = max(0, min(alpha r, alpha, beta)),
// for r = d0 / dq > 0 (the caller handles r <= 0).  min(alpha r, alpha) dq = alpha mq with
// mq = (|d0| < |dq| ? d0 : dq) = min(r, 1) dq; beta dq is bdq.  dq is the own-side difference
// (dm on the left), dother the opposite one.  alpha = clamp(alpha_t, 1, 2) with
//   alpha_t = 2 max(1, r) (1 + max(0, tt_oth / r_oth)) / (1 + tt_own),
//   tt = n / (d + S) (transverse difference over normal difference), r_oth = d0 / dother,
// and because max(1, r) mq = d0 in both cases of mq, the unclamped candidate is the single
// quotient
//   alpha_t mq = 2 (d0 (d_oth + S) + x n_oth dother) (d_own + S) / ((d_oth + S) (d_own + S + n_own))
// with x = 1 when tt_oth / r_oth > 0, else 0 (the regularisation S = 1e-30 inside the ratios
// only matters for differences below the epsilon flush).  r32, at32, b32: FP32 estimates of r,
// alpha_t and beta; bmag: the FP32 magnitude of beta's terms, which bounds the estimate's
// absolute error.  The FP32 estimates only skip work: every slope returned is a double-float
// candidate chosen by double-float comparisons, except that beta is taken without forming alpha
// when it is below alpha min(r, 1) by a margin far above the estimates' errors.
__device__ __forceinline__ df mlp_side_df(df D0, df Dq, df Dother, df n_own, df d_own, df n_oth,
                                          df d_oth, df bdq, float r32, float at32, float b32,
                                          float bmag) {
  const df mq = df_abs(D0) < df_abs(Dq) ? D0 : Dq;
  const bool pos = Dq.hi > 0.0f;
  const float mr = fminf(r32, 1.0f);
  const float a32 = fmaxf(1.0f, fminf(2.0f, at32));
  df cand;
  if (b32 < a32 * mr * (1.0f - 1e-4f) - 1e-6f * bmag - 1e-6f) {
    cand = bdq;
  } else {
    df ca;
    if (at32 >= 2.0f * (1.0f + 2e-4f)) {
      ca = df_twice(mq);
    } else if (at32 <= 1.0f - 2e-4f) {
      ca = mq;
    } else {
      const df S = df(1e-30f);
      const df ao = df_abs(d_own) + S, at = df_abs(d_oth) + S;
      const bool x = n_oth.hi != 0.0f && ((D0.hi > 0.0f) == (Dother.hi > 0.0f)) &&
                     Dother.hi != 0.0f;
      const df num = x ? D0 * at + df_abs(n_oth) * Dother : D0 * at;
      ca = df_div(df_twice(num * ao), at * (ao + df_abs(n_own)));
      // clamp alpha to [1, 2]: the candidate between mq and 2 mq (oriented by the sign of dq)
      const df m2 = df_twice(mq);
      if (pos) ca = ca < mq ? mq : (m2 < ca ? m2 : ca);
      else ca = mq < ca ? mq : (ca < m2 ? m2 : ca);
    }
    cand = pos ? (bdq < ca ? bdq : ca) : (ca < bdq ? bdq : ca);
  }
  // max(0, phi): the slope has the sign of dq, or is zero
  return pos ? (cand.hi > 0.0f ? cand : df(0.0f)) : (cand.hi < 0.0f ? cand : df(0.0f));
}

template <int ORDER>
__device__ __forceinline__ void recon_mlp_df(df qm2, df qm1, df q0, df qp1, df qp2, df qp3,
                                             df t0p, df t0m, df t1p, df t1m, df& L, df& Rr) {
  const float S = 1e-30f;
  const df Dm = flushed(q0 - qm1), D0 = flushed(qp1 - q0), Dp = flushed(qp2 - qp1);
  const float dm = Dm.hi, d0 = D0.hi, dp = Dp.hi;
  const float rR_p1 = __fdividef(d0, dp + S), rL = __fdividef(d0, dm + S);
  float bL, bR, mL, mR;  // FP32 beta estimates and the magnitudes of their terms
  df bdL, bdR;           // beta * dm (left), beta * dp (right) in double-float
  if (ORDER == 5) {
    const df Dm3 = flushed(qm1 - qm2), Dp5 = flushed(qp3 - qp2);
    const float dm3 = Dm3.hi, dp5 = Dp5.hi;
    const float rL_m1 = __fdividef(dm, dm3 + S), rL_p1 = __fdividef(dp, d0 + S);
    const float rR_p2 = __fdividef(dp, dp5 + S), rR = __fdividef(dm, d0 + S);
    const float uL = __fdividef(-2.0f, rL_m1 + S), uR = __fdividef(-2.0f, rR_p2 + S);
    bL = ((uL + 11.0f) + 24.0f * rL - 3.0f * rL * rL_p1) * (1.0f / 30.0f);
    bR = ((uR + 11.0f) + 24.0f * rR_p1 - 3.0f * rR_p1 * rR) * (1.0f / 30.0f);
    mL = (fabsf(uL) + 11.0f + 24.0f * fabsf(rL) + 3.0f * fabsf(rL * rL_p1)) * (1.0f / 30.0f);
    mR = (fabsf(uR) + 11.0f + 24.0f * fabsf(rR_p1) + 3.0f * fabsf(rR_p1 * rR)) * (1.0f / 30.0f);
    // beta_L dm = (-2 dm3 + 11 dm + 24 d0 - 3 rL rL_p1 dm)/30 with rL rL_p1 dm = dp (0 if d0 = 0)
    const df t3L = d0 == 0.0f ? df(0.0f) : Dp, t3R = d0 == 0.0f ? df(0.0f) : Dm;
    bdL = (df_scale(Dm3, -2.0f) + df_scale(Dm, 11.0f) + df_scale(D0, 24.0f) - df_scale(t3L, 3.0f)) *
          df(1.0 / 30.0);
    // beta_R dp = (-2 dp5 + 11 dp + 24 d0 - 3 rR_p1 rR dp)/30 with rR_p1 rR dp = dm
    bdR = (df_scale(Dp5, -2.0f) + df_scale(Dp, 11.0f) + df_scale(D0, 24.0f) - df_scale(t3R, 3.0f)) *
          df(1.0 / 30.0);
  } else {
    bL = (1.0f + 2.0f * rL) * (1.0f / 3.0f);
    bR = (1.0f + 2.0f * rR_p1) * (1.0f / 3.0f);
    mL = (1.0f + 2.0f * fabsf(rL)) * (1.0f / 3.0f);
    mR = (1.0f + 2.0f * fabsf(rR_p1)) * (1.0f / 3.0f);
    bdL = (Dm + df_twice(D0)) * df(1.0 / 3.0);
    bdR = (Dp + df_twice(D0)) * df(1.0 / 3.0);
  }
  // transverse ratios: numerators and denominators in double-float, FP32 estimates
  const df n0 = t0p - t0m, e0 = qp1 - qm1, n1 = t1p - t1m, e1 = qp2 - q0;
  const float tt = __fdividef(fabsf(n0.hi), fabsf(e0.hi) + S);
  const float tt1 = __fdividef(fabsf(n1.hi), fabsf(e1.hi) + S);
  const float aLt = __fdividef(2.0f * fmaxf(1.0f, rL) * (1.0f + fmaxf(0.0f, __fdividef(tt1, rR_p1 + S))),
                               1.0f + tt);
  const float aRt = __fdividef(2.0f * fmaxf(1.0f, rR_p1) * (1.0f + fmaxf(0.0f, __fdividef(tt, rL + S))),
                               1.0f + tt1);
  L = df_ratio_nonpos(D0, Dm)
          ? q0
          : q0 + df_half(mlp_side_df(D0, Dm, Dp, n0, e0, n1, e1, bdL, rL, aLt, bL, mL));
  Rr = df_ratio_nonpos(D0, Dp)
           ? qp1
           : qp1 - df_half(mlp_side_df(D0, Dp, Dm, n1, e1, n0, e0, bdR, rR_p1, aRt, bR, mR));
}

template <int ORDER>
static __device__ __noinline__ DfPair recon_mlp_df_ool(df qm2, df qm1, df q0, df qp1, df qp2,
                                                       df qp3, df t0p, df t0m, df t1p, df t1m) {
  DfPair e;
  recon_mlp_df<ORDER>(qm2, qm1, q0, qp1, qp2, qp3, t0p, t0m, t1p, t1m, e.L, e.R);
  return e;
}
template <>
__device__ __forceinline__ void recon_mlp<df, 3>(df qm2, df qm1, df q0, df qp1, df qp2, df qp3,
                                                 df t0p, df t0m, df t1p, df t1m, df& L, df& Rr) {
  const DfPair e = recon_mlp_df_ool<3>(qm2, qm1, q0, qp1, qp2, qp3, t0p, t0m, t1p, t1m);
  L = e.L;
  Rr = e.R;
}
template <>
__device__ __forceinline__ void recon_mlp<df, 5>(df qm2, df qm1, df q0, df qp1, df qp2, df qp3,
                                                 df t0p, df t0m, df t1p, df t1m, df& L, df& Rr) {
  const DfPair e = recon_mlp_df_ool<5>(qm2, qm1, q0, qp1, qp2, qp3, t0p, t0m, t1p, t1m);
  L = e.L;
  Rr = e.R;
}

// ---------------------------------------------------------------------------------------------
// Edge fluxes.  DIR = 0: i-edge (normal x, n = (1,0)); DIR = 1: j-edge (normal y, n = (0,1)).
// The Cartesian normals are exact (quad_cell.f90:193-229 on axis-aligned cells), so the
// reference's products with n_x / n_y are folded: x*1 = x and x*0 + y = y exactly.
// Cell-pressure stencils for the shock sensors are given in edge-local coordinates:
// pc(n, t) = cell at normal offset n (0 = left cell, 1 = right cell) and tangential offset t.
// ---------------------------------------------------------------------------------------------
template <typename R> struct FluxConsts {
  R gamma, g_over_gm1, gm1, two_gm1_over_gp1, gamma_factor, hllc_gf, harten_delta;
  R ausm_beta, ausm_kp, ausm_ku, ausm_sigma;
  int low_mach_fix, harten;
};

// The FP64 constants carried to another compute type (host side).
template <typename R> inline FluxConsts<R> convert_consts(const FluxConsts<double>& K) {
  FluxConsts<R> C{};
  C.gamma = R(K.gamma);
  C.g_over_gm1 = R(K.g_over_gm1);
  C.gm1 = R(K.gm1);
  C.two_gm1_over_gp1 = R(K.two_gm1_over_gp1);
  C.gamma_factor = R(K.gamma_factor);
  C.hllc_gf = R(K.hllc_gf);
  C.harten_delta = R(K.harten_delta);
  C.ausm_beta = R(K.ausm_beta);
  C.ausm_kp = R(K.ausm_kp);
  C.ausm_ku = R(K.ausm_ku);
  C.ausm_sigma = R(K.ausm_sigma);
  C.low_mach_fix = K.low_mach_fix;
  C.harten = K.harten;
  return C;
}

template <typename R> struct Prim { R r, u, v, p; };

// AUSMPW+ split functions, ausmpw_plus_solver.fypp:486-530 (alpha = 1/8)
template <typename R> __device__ __forceinline__ R aw_p_plus(R M) {
  if (rabs(M) > R(1)) return half(R(1) + fsign1(M));
  return quarter((M + R(1)) * (M + R(1))) * (R(2) - M) +
         eighth(M) * ((M * M - R(1)) * (M * M - R(1)));
}
template <typename R> __device__ __forceinline__ R aw_p_minus(R M) {
  if (rabs(M) > R(1)) return half(R(1) - fsign1(M));
  return quarter((M - R(1)) * (M - R(1))) * (R(2) + M) -
         eighth(M) * ((M * M - R(1)) * (M * M - R(1)));
}
template <typename R> __device__ __forceinline__ R aw_m_plus(R M) {
  if (rabs(M) > R(1)) return half(M + rabs(M));
  return quarter((M + R(1)) * (M + R(1)));
}
template <typename R> __device__ __forceinline__ R aw_m_minus(R M) {
  if (rabs(M) > R(1)) return half(M - rabs(M));
  return -quarter((M - R(1)) * (M - R(1)));
}

// AUSMPW+, ausmpw_plus_solver.fypp:336-459.  pc[4] = p1_L, p1_R, p2_L, p2_R (:430-442).
template <typename R, int DIR>
__device__ __forceinline__ void flux_ausmpw(const FluxConsts<R>& K, const Prim<R>& A,
                                            const Prim<R>& B, const R pc[4], R F[4]) {
  const R g = R(K.gamma);
  R rho_L = A.r, u_LHS = A.u, v_LHS = A.v, p_L = A.p;
  R rho_R = B.r, u_RHS = B.u, v_RHS = B.v, p_R = B.p;
  const R U_L = DIR == 0 ? u_LHS : v_LHS, U_R = DIR == 0 ? u_RHS : v_RHS;
  const R V_L = DIR == 0 ? v_LHS : u_LHS, V_R = DIR == 0 ? v_RHS : u_RHS;
  R cs_L = Num<R>::sqrt(Num<R>::div(g * p_L, rho_L));
  R cs_R = Num<R>::sqrt(Num<R>::div(g * p_R, rho_R));
  R M_LHS = Num<R>::div(Num<R>::sqrt(u_LHS * u_LHS + v_LHS * v_LHS), cs_L);
  R M_RHS = Num<R>::div(Num<R>::sqrt(u_RHS * u_RHS + v_RHS * v_RHS), cs_R);
  if (K.low_mach_fix && (rabs(M_LHS) < R(0.1) || rabs(M_RHS) < R(0.1))) {  // LOW_MACH
    R f_M = rmin(R(1), rmax(M_LHS, M_RHS));
    R uLf = half(u_LHS + u_RHS) + half(f_M) * (u_LHS - u_RHS);
    R uRf = half(u_LHS + u_RHS) - half(f_M) * (u_LHS - u_RHS);
    R vLf = half(v_LHS + v_RHS) + half(f_M) * (v_LHS - v_RHS);
    R vRf = half(v_LHS + v_RHS) - half(f_M) * (v_LHS - v_RHS);
    u_LHS = uLf; u_RHS = uRf; v_LHS = vLf; v_RHS = vRf;
  }
  const R gg = R(K.g_over_gm1);
  R H_L = gg * Num<R>::div(p_L, rho_L) + half(u_LHS * u_LHS + v_LHS * v_LHS);
  R H_R = gg * Num<R>::div(p_R, rho_R) + half(u_RHS * u_RHS + v_RHS * v_RHS);
  R H_normal = rmin(H_L - half(V_L * V_L), H_R - half(V_R * V_R));
  R c_s = Num<R>::sqrt(R(K.two_gm1_over_gp1) * H_normal);
  R c_half;
  if (half(U_L + U_R) < R(0)) c_half = Num<R>::div(c_s * c_s, rmax(rabs(U_R), c_s));
  else c_half = Num<R>::div(c_s * c_s, rmax(rabs(U_L), c_s));
  R M_L = Num<R>::div(U_L, c_half);
  R M_R = Num<R>::div(U_R, c_half);
  R M_L_plus = aw_m_plus(M_L);
  R M_R_minus = aw_m_minus(M_R);
  R P_R_minus = aw_p_minus(M_R);
  R P_L_plus = aw_p_plus(M_L);
  R p_s = p_L * P_L_plus + p_R * P_R_minus;
  R mt = rmin(Num<R>::div(p_L, p_R), Num<R>::div(p_R, p_L));
  R w = R(1) - mt * mt * mt;
  R f_L, f_R;
  if (abs_lt(p_s, Num<R>::tiny)) {
    f_L = R(0);
    f_R = R(0);
  } else {
    R t = rmin(R(1), Num<R>::div(rmin(rmin(rmin(pc[0], pc[1]), pc[2]), pc[3]), rmin(p_L, p_R)));
    R min_term = t * t;
    f_L = (Num<R>::div(p_L, p_s) - R(1)) * min_term;
    f_R = (Num<R>::div(p_R, p_s) - R(1)) * min_term;
  }
  R Mb_L, Mb_R;
  if (M_L_plus + M_R_minus < R(0)) {
    Mb_L = M_L_plus * w * (R(1) + f_L);
    Mb_R = M_R_minus + M_L_plus * ((R(1) - w) * (R(1) + f_L) - f_R);
  } else {
    Mb_L = M_L_plus + M_R_minus * ((R(1) - w) * (R(1) + f_R) - f_L);
    Mb_R = M_R_minus * w * (R(1) + f_R);
  }
  R mL = Mb_L * c_half * rho_L;
  R mR = Mb_R * c_half * rho_R;
  F[0] = mL + mR;
  // pressure terms carry n_x = 1 (DIR 0) or n_y = 1 (DIR 1); the other is an exact zero
  R pterm = (P_L_plus * p_L) + (P_R_minus * p_R);
  if (DIR == 0) {
    F[1] = (mL * u_LHS) + (mR * u_RHS) + pterm;
    F[2] = (mL * v_LHS) + (mR * v_RHS) + ((P_L_plus * R(0) * p_L) + (P_R_minus * R(0) * p_R));
  } else {
    F[1] = (mL * u_LHS) + (mR * u_RHS) + ((P_L_plus * R(0) * p_L) + (P_R_minus * R(0) * p_R));
    F[2] = (mL * v_LHS) + (mR * v_RHS) + pterm;
  }
  F[3] = (mL * H_L) + (mR * H_R);
}

// M-AUSMPW+, the active code of m_ausmpw_plus_solver.fypp:437-708: AUSMPW+'s interface Mach
// number and w sensor, pressure splitting without the alpha term (:600-610), the shock sensor f
// with 1e-10 cuts (get_f, :804-843), interface states blended towards the superbee edge states
// (phi_L_half / phi_R_half, :768-800; As, Bs) and flux cuts at epsilon*1e3 (:369, :684-705).
// U_L/U_R/V_L/V_R are taken before the low-Mach fix, as in the reference.
template <typename R>
__device__ __forceinline__ R mausm_p_plus(R M) {
  if (rabs(M) > R(1)) return half(R(1) + fsign1(M));
  return quarter((M + R(1)) * (M + R(1))) * (R(2) - M);
}
template <typename R>
__device__ __forceinline__ R mausm_p_minus(R M) {
  if (rabs(M) > R(1)) return half(R(1) - fsign1(M));
  return quarter((M - R(1)) * (M - R(1))) * (R(2) + M);
}
template <typename R>
__device__ __forceinline__ R mausm_phi_L(R pL, R pR, R pLsb, R a) {
  if (rabs(pR - pL) < R(1) || rabs(pLsb - pL) < Num<R>::eps) return pL;
  return pL + Num<R>::div(rmax(R(0), (pR - pL) * (pLsb - pL)), (pR - pL) * rabs(pLsb - pL)) *
                  rmin(rmin(a, half(rabs(pR - pL))), rabs(pLsb - pL));
}
template <typename R>
__device__ __forceinline__ R mausm_phi_R(R pL, R pR, R pRsb, R a) {
  if (rabs(pL - pR) < Num<R>::eps || rabs(pRsb - pR) < R(1)) return pR;
  return pR + Num<R>::div(rmax(R(0), (pL - pR) * (pRsb - pR)), (pL - pR) * rabs(pRsb - pR)) *
                  rmin(rmin(a, half(rabs(pL - pR))), rabs(pRsb - pR));
}

template <typename R, int DIR>
__device__ __forceinline__ void flux_mausmpw(const FluxConsts<R>& K, const Prim<R>& A,
                                             const Prim<R>& B, const Prim<R>& As,
                                             const Prim<R>& Bs, const R pc[4], R F[4]) {
  const R g = R(K.gamma);
  const R EPSF = R(2.220446049250313080847263336181640625e-13);  // epsilon(1.0_rk) * 1e3_rk
  const R CUT = R(1e-10);
  R rho_L = A.r, u_LHS = A.u, v_LHS = A.v, p_L = A.p;
  R rho_R = B.r, u_RHS = B.u, v_RHS = B.v, p_R = B.p;
  const R U_L = DIR == 0 ? u_LHS : v_LHS, U_R = DIR == 0 ? u_RHS : v_RHS;
  const R V_L = DIR == 0 ? v_LHS : u_LHS, V_R = DIR == 0 ? v_RHS : u_RHS;
  R cs_L = Num<R>::sqrt(Num<R>::div(g * p_L, rho_L));
  R cs_R = Num<R>::sqrt(Num<R>::div(g * p_R, rho_R));
  R M_LHS = Num<R>::div(Num<R>::sqrt(u_LHS * u_LHS + v_LHS * v_LHS), cs_L);
  R M_RHS = Num<R>::div(Num<R>::sqrt(u_RHS * u_RHS + v_RHS * v_RHS), cs_R);
  if (K.low_mach_fix && (rabs(M_LHS) < R(0.1) || rabs(M_RHS) < R(0.1))) {  // LOW_MACH
    R f_M = rmin(R(1), rmax(M_LHS, M_RHS));
    R uLf = half(u_LHS + u_RHS) + half(f_M) * (u_LHS - u_RHS);
    R uRf = half(u_LHS + u_RHS) - half(f_M) * (u_LHS - u_RHS);
    R vLf = half(v_LHS + v_RHS) + half(f_M) * (v_LHS - v_RHS);
    R vRf = half(v_LHS + v_RHS) - half(f_M) * (v_LHS - v_RHS);
    u_LHS = uLf; u_RHS = uRf; v_LHS = vLf; v_RHS = vRf;
  }
  const R gg = R(K.g_over_gm1);
  R H_L = gg * Num<R>::div(p_L, rho_L) + half(u_LHS * u_LHS + v_LHS * v_LHS);
  R H_R = gg * Num<R>::div(p_R, rho_R) + half(u_RHS * u_RHS + v_RHS * v_RHS);
  R H_normal = rmin(H_L - half(V_L * V_L), H_R - half(V_R * V_R));
  R c_s = Num<R>::sqrt(R(K.two_gm1_over_gp1) * H_normal);
  R c_half;
  if (half(U_L + U_R) < R(0)) c_half = Num<R>::div(c_s * c_s, rmax(rabs(U_R), c_s));
  else c_half = Num<R>::div(c_s * c_s, rmax(rabs(U_L), c_s));
  R M_L = Num<R>::div(U_L, c_half);
  R M_R = Num<R>::div(U_R, c_half);
  R M_L_plus = aw_m_plus(M_L);
  R M_R_minus = aw_m_minus(M_R);
  R P_R_minus = mausm_p_minus(M_R);
  R P_L_plus = mausm_p_plus(M_L);
  R p_s = p_L * P_L_plus + p_R * P_R_minus;
  R mt = rmin(Num<R>::div(p_L, p_R), Num<R>::div(p_R, p_L));
  R w = R(1) - (mt * mt * mt);
  R f_L, f_R;
  if (abs_lt(p_s, Num<R>::tiny)) {
    f_L = R(0);
    f_R = R(0);
  } else {
    R t = rmin(R(1), Num<R>::div(rmin(rmin(rmin(pc[0], pc[1]), pc[2]), pc[3]), rmin(p_L, p_R)));
    R min_term = t * t;
    if (rabs(R(1) - min_term) < CUT) min_term = R(1);
    R fl = Num<R>::div(p_L, p_s) - R(1);
    if (rabs(fl) < CUT) fl = R(0);
    f_L = fl * min_term;
    R fr = Num<R>::div(p_R, p_s) - R(1);
    if (rabs(fr) < CUT) fr = R(0);
    f_R = fr * min_term;
  }
  R Mb_L, Mb_R;
  if (M_L_plus + M_R_minus < R(0)) {
    Mb_L = M_L_plus * w * (R(1) + f_L);
    Mb_R = M_R_minus + M_L_plus * ((R(1) - w) * (R(1) + f_L) - f_R);
  } else {
    Mb_L = M_L_plus + M_R_minus * ((R(1) - w) * (R(1) + f_R) - f_L);
    Mb_R = M_R_minus * w * (R(1) + f_R);
  }
  R t2 = rmin(R(1), rmax(rabs(M_L), rabs(M_R)));
  R a = R(1) - t2 * t2;
  R rLh = mausm_phi_L(rho_L, rho_R, As.r, a), rRh = mausm_phi_R(rho_L, rho_R, Bs.r, a);
  R uLh = mausm_phi_L(u_LHS, u_RHS, As.u, a), uRh = mausm_phi_R(u_LHS, u_RHS, Bs.u, a);
  R vLh = mausm_phi_L(v_LHS, v_RHS, As.v, a), vRh = mausm_phi_R(v_LHS, v_RHS, Bs.v, a);
  R pLh = mausm_phi_L(p_L, p_R, As.p, a), pRh = mausm_phi_R(p_L, p_R, Bs.p, a);
  R H_Lh = gg * Num<R>::div(pLh, rLh) + half(uLh * uLh + vLh * vLh);
  R H_Rh = gg * Num<R>::div(pRh, rRh) + half(uRh * uRh + vRh * vRh);
  R mL = Mb_L * c_half * rLh;
  R mR = Mb_R * c_half * rRh;
  if (rabs(mL + mR) < EPSF) { mL = R(0); mR = R(0); }
  F[0] = mL + mR;
  // pressure terms carry n_x = 1 (DIR 0) or n_y = 1 (DIR 1); the other is an exact zero
  const R pn = (P_L_plus * p_L) + (P_R_minus * p_R);
  const R pz = (P_L_plus * R(0) * p_L) + (P_R_minus * R(0) * p_R);
  const R px = DIR == 0 ? pn : pz, py = DIR == 0 ? pz : pn;
  const R tx = (mL * uLh) + (mR * uRh), ty = (mL * vLh) + (mR * vRh);
  F[1] = rabs(tx) < EPSF ? px : tx + px;
  F[2] = rabs(ty) < EPSF ? py : ty + py;
  F[3] = (mL * H_Lh) + (mR * H_Rh);
  if (rabs(F[3]) < EPSF) F[3] = R(0);
}

// SLAU / SLAU2 / SD-SLAU / SD-SLAU2, slau_solver.fypp:332-490.  dpair[6][2]: delta_p1..6 cells.
template <typename R, int DIR, int VARIANT>
__device__ __forceinline__ void flux_slau(const FluxConsts<R>& K, const Prim<R>& A, const Prim<R>& B,
                                          const R dpa[6], const R dpb[6], R F[4]) {
  const R g = R(K.gamma);
  const R EPS = Num<R>::eps;
  const R THRESHOLD = R(5e-3), C_SD1 = R(0.01);
  R rho_L = A.r, u_L = A.u, v_L = A.v, p_L = A.p;
  R rho_R = B.r, u_R = B.u, v_R = B.v, p_R = B.p;
  // V_n = u*n_x + v*n_y with an exact unit normal
  R Vp = DIR == 0 ? add_mul0(u_L, v_L) : add_mul0(v_L, u_L);
  R Vm = DIR == 0 ? add_mul0(u_R, v_R) : add_mul0(v_R, u_R);
  R c_plus = Num<R>::sqrt(Num<R>::div(g * p_L, rho_L));
  R c_minus = Num<R>::sqrt(Num<R>::div(g * p_R, rho_R));
  R c_bar = half(c_plus + c_minus);
  R V_n_bar = Num<R>::div(rho_L * rabs(Vp) + rho_R * rabs(Vm), rho_L + rho_R);
  R vel2 = half(u_L * u_L + v_L * v_L + u_R * u_R + v_R * v_R);
  R M_hat = rmin(R(1), Num<R>::div(Num<R>::sqrt(vel2), c_bar));
  R M_bar = Num<R>::div(V_n_bar, c_bar);
  R M_plus = Num<R>::div(Vp, c_bar);
  R M_minus = Num<R>::div(Vm, c_bar);
  R Chi = (R(1) - M_hat) * (R(1) - M_hat);
  R p_bar = half(p_L + p_R);
  R rho_bar = half(rho_L + rho_R);
  R B_plus, B_minus;
  if (rabs(M_plus) < R(1)) B_plus = quarter(R(2) - M_plus) * ((M_plus + R(1)) * (M_plus + R(1)));
  else B_plus = half(R(1) + fsign1(M_plus));
  if (rabs(M_minus) < R(1))
    B_minus = quarter(R(2) + M_minus) * ((M_minus - R(1)) * (M_minus - R(1)));
  else B_minus = half(R(1) + fsign1(-M_minus));
  R delta_p = p_R - p_L;
  if (abs_lt(delta_p, EPS) || rabs(delta_p) < THRESHOLD * p_bar) delta_p = R(0);
  R delta_rho = rho_R - rho_L;
  if (abs_lt(delta_rho, EPS)) delta_rho = R(0);
  R delta_B = B_plus - B_minus;
  if (abs_lt(delta_B, EPS)) delta_B = R(0);
  R pLmR = p_L - p_R;
  if (abs_lt(pLmR, EPS)) pLmR = R(0);
  R theta = R(0);
  if (VARIANT == FLUX_SD_SLAU || VARIANT == FLUX_SD_SLAU2) {
    R m6 = R(0);
    R dpk[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      dpk[k] = rabs(dpa[k] - dpb[k]);
      if (dpk[k] < EPS || dpk[k] < THRESHOLD * p_bar) dpk[k] = R(0);
    }
    m6 = rmax(rmax(rmax(rmax(rmax(dpk[0], dpk[1]), dpk[2]), dpk[3]), dpk[4]), dpk[5]);
    R dp_max = rmax(rabs(delta_p), m6);
    R ratio = Num<R>::div(Num<R>::div(C_SD1 * rabs(delta_p), p_bar) + C_SD1,
                          Num<R>::div(dp_max, p_bar) + C_SD1);
    theta = rmin(R(1), ratio * ratio) * rmax(R(0), R(1) - rabs(M_bar));
  }
  R p_tilde;
  if (VARIANT == FLUX_SLAU || VARIANT == FLUX_SD_SLAU)
    p_tilde = (p_bar + half(delta_B) * pLmR) + (R(1) - Chi) * (B_plus + B_minus - R(1)) * p_bar;
  else
    p_tilde = p_bar + (half(delta_B) * pLmR) +
              Num<R>::sqrt(vel2) * (B_plus + B_minus - R(1)) * rho_bar * c_bar;
  R gg = -(rmax(rmin(M_plus, R(0)), R(-1)) * rmin(rmax(M_minus, R(0)), R(1)));
  R diss = (VARIANT == FLUX_SLAU || VARIANT == FLUX_SLAU2) ? Chi : theta;
  R mf = half((rho_L * Vp) + (rho_R * Vm) - rabs(V_n_bar) * delta_rho) * (R(1) - gg) -
         (Num<R>::div(diss, twice(c_bar)) * delta_p);
  R mL = half(mf + rabs(mf));
  R mR = half(mf - rabs(mf));
  const R gq = R(K.g_over_gm1);
  R H_L = gq * Num<R>::div(p_L, rho_L) + half(u_L * u_L + v_L * v_L);
  R H_R = gq * Num<R>::div(p_R, rho_R) + half(u_R * u_R + v_R * v_R);
  F[0] = mL + mR;
  if (DIR == 0) {
    F[1] = (mL * u_L) + (mR * u_R) + p_tilde;
    F[2] = add_mul0((mL * v_L) + (mR * v_R), p_tilde);
  } else {
    F[1] = add_mul0((mL * u_L) + (mR * u_R), p_tilde);
    F[2] = (mL * v_L) + (mR * v_R) + p_tilde;
  }
  F[3] = (mL * H_L) + (mR * H_R);
}

// Roe with the reference's wave-speed bounds and pressure-sensor shear correction,
// roe_solver.fypp:420-512; optional Harten fix (:529-536).  fh: the five f_h pairs (:495-508).
template <typename R, int DIR>
__device__ __forceinline__ void flux_roe(const FluxConsts<R>& K, const Prim<R>& A, const Prim<R>& B,
                                         const R fa[5], const R fb[5], R F[4]) {
  // products through Num<R>::mul (the integer pipe on the FP64 path), in the same left-to-right
  // order as the expressions they spell out
  auto m = [](R x, R y) { return Num<R>::mul(x, y); };
  const R g = R(K.gamma);
  R rl = rabs(A.r), ul = A.u, vl = A.v, pl = rabs(A.p);
  R rr = rabs(B.r), ur = B.u, vr = B.v, pr = rabs(B.p);
  const R gq = R(K.g_over_gm1);
  R rav = Num<R>::sqrt(m(rl, rr));
  R q_pl = Num<R>::div(pl, rl), q_rav = Num<R>::div(rav, rl), q_gpl = Num<R>::div(m(g, pl), rl);
  R hl = m(gq, q_pl) + half(m(ul, ul) + m(vl, vl));
  R hr = m(gq, Num<R>::div(pr, rr)) + half(m(ur, ur) + m(vr, vr));
  R gam1 = R(K.gm1);
  R dd = q_rav;
  R dd1 = Num<R>::div(R(1), R(1) + dd);
  R uav = m(ul + m(dd, ur), dd1);
  R vav = m(vl + m(dd, vr), dd1);
  R hav = m(hl + m(dd, hr), dd1);
  R q2a = half(m(uav, uav) + m(vav, vav));
  R c2a = m(gam1, hav - q2a);
  R cav = Num<R>::sqrt(c2a);
  // x n_x + y n_y with the unit normal's exact 1 and 0 (a product with 1 is the operand)
  auto dotn = [](R x, R y) { return DIR == 0 ? add_mul0(x, y) : add_mul0(y, x); };
  R uv = dotn(uav, vav);
  R du = dotn(ur - ul, vr - vl);
  R du_trans = DIR == 0 ? add_mul0(vr - vl, -(ur - ul)) : add_mul0(-(ur - ul), vr - vl);
  R cs_R = Num<R>::sqrt(Num<R>::div(m(g, pr), rr));
  R cs_L = Num<R>::sqrt(q_gpl);
  R h1 = rabs(rmin(uv - cav, dotn(ul, vl) - cs_L));
  R h2 = rabs(uv);
  R h4 = rabs(rmax(uv + cav, dotn(ur, vr) + cs_R));
  R e1 = h1, e2 = h2, e4 = h4;
  if (K.harten) {
    R delta = m(R(K.harten_delta), cav);
    e1 = (h1 > delta) ? h1 : Num<R>::div(half(m(h1, h1) + m(delta, delta)), delta);
    e2 = (h2 > delta) ? h2 : Num<R>::div(half(m(h2, h2) + m(delta, delta)), delta);
    e4 = (h4 > delta) ? h4 : Num<R>::div(half(m(h4, h4) + m(delta, delta)), delta);
  }
  h1 = m(m(rav, cav), du);
  h2 = Num<R>::div(m(e1, pr - pl - h1), twice(c2a));
  R h3 = m(e2, rr - rl - Num<R>::div(pr - pl, c2a));
  h4 = m(e2, rav);
  R h5 = Num<R>::div(m(e4, pr - pl + h1), twice(c2a));
  R psi = Num<R>::div(rabs(cs_R - cs_L), rmax(cs_R, cs_L));
  // the normal-direction terms carry the exact 1, the tangential ones the exact 0
  auto on = [](bool axis, R a, R b) { return axis ? a + b : add_mul0(a, b); };
  R FR0 = m(rr, uv), FR1 = on(DIR == 0, m(m(rr, ur), uv), pr), FR2 = on(DIR == 1, m(m(rr, vr), uv), pr);
  R FR3 = m(m(rr, hr), uv);
  R FL0 = m(rl, uv), FL1 = on(DIR == 0, m(m(rl, ul), uv), pl), FL2 = on(DIR == 1, m(m(rl, vl), uv), pl);
  R FL3 = m(m(rl, hl), uv);
  R m0 = (h2 + h3 + h5);
  R m1 = (m(h2, on(DIR == 0, uav, -cav)) + m(h3, uav) + m(h4, on(DIR == 0, ur - ul, -du)) +
          m(h5, on(DIR == 0, uav, cav)));
  R m2 = (m(h2, on(DIR == 1, vav, -cav)) + m(h3, vav) + m(h4, on(DIR == 1, vr - vl, -du)) +
          m(h5, on(DIR == 1, vav, cav)));
  R m3 = (m(h2, hav - m(cav, uv)) + m(h3, q2a) +
          m(h4, m(uav, ur - ul) + m(vav, vr - vl) - m(uv, du)) + m(h5, hav + m(cav, uv)));
  F[0] = half(FR0 + FL0 - m0);
  F[1] = half(FR1 + FL1 - m1);
  F[2] = half(FR2 + FL2 - m2);
  F[3] = half(FR3 + FL3 - m3);
  R fmax = R(0);
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    R ratio = Num<R>::div(rabs(fb[k] - fa[k]), rmin(fb[k], fa[k]) + R(1e-16));
    fmax = rmax(fmax, (ratio < R(1)) ? R(0) : R(1));
  }
  // -(du_trans n_y) + psi du n_x and du_trans n_x + psi du n_y
  const R c1 = DIR == 0 ? add_mul0(m(psi, du), -du_trans) : add_mul0(-du_trans, m(psi, du));
  const R c2 = DIR == 0 ? add_mul0(du_trans, m(psi, du)) : add_mul0(m(psi, du), du_trans);
  F[1] = F[1] - m(m(m(half(fmax), rav), cav), c1);
  F[2] = F[2] - m(m(m(half(fmax), rav), cav), c2);
}

// AUSM+-up (basic), ausm_plus_solver.f90:499-643 + upwinding of the commented driver :313-325.
template <typename R> __device__ __forceinline__ R up_m1p(R M) { return half(M + rabs(M)); }
template <typename R> __device__ __forceinline__ R up_m1m(R M) { return half(M - rabs(M)); }
template <typename R> __device__ __forceinline__ R up_m2p(R M) { return quarter((M + R(1)) * (M + R(1))); }
template <typename R> __device__ __forceinline__ R up_m2m(R M) { return -quarter((M - R(1)) * (M - R(1))); }

template <typename R, int DIR>
__device__ __forceinline__ void flux_ausm_up(const FluxConsts<R>& K, const Prim<R>& A,
                                             const Prim<R>& B, R F[4]) {
  const R EPS = Num<R>::eps;
  const R alpha = R(3.0 / 16.0);
  const R gamma_factor = R(K.gamma_factor);
  R vel_L = DIR == 0 ? add_mul0(A.u, A.v) : add_mul0(A.v, A.u);
  R vel_R = DIR == 0 ? add_mul0(B.u, B.v) : add_mul0(B.v, B.u);
  const R gq = R(K.g_over_gm1);
  R H_L = Num<R>::div(A.p, A.r) * gq + half(A.u * A.u + A.v * A.v);
  R H_R = Num<R>::div(B.p, B.r) * gq + half(B.u * B.u + B.v * B.v);
  R a_crit_L = Num<R>::sqrt(gamma_factor * rabs(H_L));
  R a_crit_R = Num<R>::sqrt(gamma_factor * rabs(H_R));
  R a_circ_L = Num<R>::div(a_crit_L * a_crit_L, rmax(a_crit_L, vel_L));
  R a_circ_R = Num<R>::div(a_crit_R * a_crit_R, rmax(a_crit_R, -vel_R));
  R a_half = rmin(a_circ_L, a_circ_R);
  R M_L = Num<R>::div(vel_L, a_half);
  R M_R = Num<R>::div(vel_R, a_half);
  R M_bar_sq = half(M_L + M_R);  // as written at ausm_plus_solver.f90:585
  const R beta = R(K.ausm_beta);
  R M_plus = (rabs(M_L) >= R(1)) ? up_m1p(M_L) : up_m2p(M_L) * (R(1) - R(16) * beta * up_m2m(M_L));
  R M_minus = (rabs(M_R) >= R(1)) ? up_m1m(M_R) : up_m2m(M_R) * (R(1) + R(16) * beta * up_m2p(M_R));
  R rho_half = half(B.r + A.r);
  R M_p;
  if (abs_lt(B.p - A.p, EPS)) M_p = R(0);
  else
    M_p = -(R(K.ausm_kp) * rmax(R(1) - R(K.ausm_sigma) * M_bar_sq, R(0)) *
            Num<R>::div(B.p - A.p, rho_half * (a_half * a_half)));
  R M_sum = M_plus + M_minus;
  if (abs_lt(M_sum, R(1e-13))) M_sum = R(0);
  R M_half = M_sum + M_p;
  if (abs_lt(M_half, R(1e-13))) M_half = R(0);
  R P_plus = (rabs(M_L) >= R(1)) ? Num<R>::div(up_m1p(M_L), M_L)
                                 : up_m2p(M_L) * ((R(2) - M_L) - R(16) * alpha * M_L * up_m2m(M_L));
  R P_minus = (rabs(M_R) >= R(1)) ? Num<R>::div(up_m1m(M_R), M_R)
                                  : up_m2m(M_R) * ((R(-2) - M_R) + R(16) * alpha * M_R * up_m2p(M_R));
  R p_u;
  if (abs_lt(vel_R - vel_L, EPS)) p_u = R(0);
  else p_u = -(R(K.ausm_ku) * P_plus * P_minus * (A.r + B.r) * a_half * (vel_R - vel_L));
  R p_half = P_plus * A.p + P_minus * B.p + p_u;
  const bool left = M_half > R(0);
  const Prim<R>& S = left ? A : B;
  R H = left ? H_L : H_R;
  R mf = M_half * a_half * S.r;
  F[0] = mf;
  F[1] = mf * S.u + (DIR == 0 ? p_half : R(0) * p_half);
  F[2] = mf * S.v + (DIR == 0 ? R(0) * p_half : p_half);
  F[3] = mf * H;
}

// HLLC (Toro 2009, Sec. 10.4-10.6) with PVRS pressure-based wave speeds; the reference's
// hllc_solver.fypp is an unfinished stub, so this follows the published method.
template <typename R, int DIR>
__device__ __forceinline__ void flux_hllc(const FluxConsts<R>& K, const Prim<R>& A, const Prim<R>& B,
                                          R F[4]) {
  // products through Num<R>::mul: on the FP64 path they run on the integer pipe (mul_rn), in the
  // same left-to-right order as the expressions they spell out
  auto m = [](R x, R y) { return Num<R>::mul(x, y); };
  const R g = R(K.gamma);
  R qnL = DIR == 0 ? A.u : A.v, qtL = DIR == 0 ? A.v : A.u;
  R qnR = DIR == 0 ? B.u : B.v, qtR = DIR == 0 ? B.v : B.u;
  R cL = Num<R>::sqrt(Num<R>::div(m(g, A.p), A.r)), cR = Num<R>::sqrt(Num<R>::div(m(g, B.p), B.r));
  R rho_bar = half(A.r + B.r), c_bar = half(cL + cR);
  R p_pvrs = half(A.p + B.p) - m(m(half(qnR - qnL), rho_bar), c_bar);
  R p_star = rmax(R(0), p_pvrs);
  const R gf = R(K.hllc_gf);
  // SL = qnL - cL qL, SR = qnR + cR qR with q = 1 (then c q is c) unless p_star exceeds p
  R SL, SR;
  if (le(p_star, A.p)) SL = qnL - cL;
  else SL = qnL - m(cL, Num<R>::sqrt(R(1) + m(gf, Num<R>::div(p_star, A.p) - R(1))));
  if (le(p_star, B.p)) SR = qnR + cR;
  else SR = qnR + m(cR, Num<R>::sqrt(R(1) + m(gf, Num<R>::div(p_star, B.p) - R(1))));
  // the total energy of the side the flux is taken from (only that one is needed)
  auto energy = [&](const Prim<R>& S) {
    return Num<R>::div(S.p, R(K.gm1)) + m(half(S.r), m(S.u, S.u) + m(S.v, S.v));
  };
  R S_star = Num<R>::div(B.p - A.p + m(m(A.r, qnL), SL - qnL) - m(m(B.r, qnR), SR - qnR),
                         m(A.r, SL - qnL) - m(B.r, SR - qnR));
  R Fn[4];
  if (ge0(SL) || !(gt0(SR) || ge0(S_star))) {
    const bool useL = ge0(SL);
    const Prim<R>& S = useL ? A : B;
    R qn = useL ? qnL : qnR, qt = useL ? qtL : qtR, E = energy(S);
    const R rq = m(S.r, qn);
    Fn[0] = rq;
    Fn[1] = m(rq, qn) + S.p;
    Fn[2] = m(rq, qt);
    Fn[3] = m(qn, E + S.p);
  } else {
    const bool useL = ge0(S_star);
    const Prim<R>& S = useL ? A : B;
    R qn = useL ? qnL : qnR, qt = useL ? qtL : qtR, E = energy(S), SK = useL ? SL : SR;
    const R rk = m(S.r, SK - qn);
    R f = Num<R>::div(rk, SK - S_star);
    R Us0 = f, Us1 = m(f, S_star), Us2 = m(f, qt);
    R Us3 = m(f, Num<R>::div(E, S.r) + m(S_star - qn, S_star + Num<R>::div(S.p, rk)));
    const R rq = m(S.r, qn);
    Fn[0] = rq + m(SK, Us0 - S.r);
    Fn[1] = (m(rq, qn) + S.p) + m(SK, Us1 - rq);
    Fn[2] = m(rq, qt) + m(SK, Us2 - m(S.r, qt));
    Fn[3] = m(qn, E + S.p) + m(SK, Us3 - E);
  }
  F[0] = Fn[0];
  F[1] = DIR == 0 ? Fn[1] : Fn[2];
  F[2] = DIR == 0 ? Fn[2] : Fn[1];
  F[3] = Fn[3];
}

// ---------------------------------------------------------------------------------------------
// flux_split_edges for one cell and one conserved variable, flux_solver.f90:252-425.
// ---------------------------------------------------------------------------------------------
constexpr int kNotPow2 = 1 << 20;

struct Geom {
  double vol, l1, l2, l3, l4;  // volume, edge lengths (bottom, right, top, left)
  double dx, dy;               // min_dx / min_dy for the CFL step
  double inv_vol;              // 1/vol when vol is a power of two (x/vol == x*inv_vol exactly), else 0
  // base-2 exponents of l1..l4 and inv_vol when they are powers of two, else kNotPow2: the
  // products with them are exponent steps
  int k1 = kNotPow2, k2 = kNotPow2, k3 = kNotPow2, k4 = kNotPow2, kinv = kNotPow2;
  // Rectilinear grids (null pointers on a uniform grid): per column i the cell width
  // x(i+1) - x(i), its edge length and reciprocal; per row j the same in y.  Every pycato grid
  // (uniform and layered, generate_initial_grids.py) is a tensor product of 1-D node arrays.
  const double* dxc;
  const double* lxc;
  const double* rdxc;
  const float* rdxf;
  const double* dyc;
  const double* lyc;
  const double* rdyc;
  const float* rdyf;
};

// quad_cell_t metrics of interior cell (i, j) (0-based) of a rectilinear grid, with the formulas
// of quad_cell.f90 on the cell's four corners (x_i, y_j) .. (x_i+1, y_j+1): volume
// dx dy - 0 * 0, edge lengths lx, ly, lx, ly snapped to the largest when they differ by
// < 2 eps, min_dx = dx, min_dy = dy.  A uniform grid returns its constant metrics.
__device__ __forceinline__ Geom cell_geom(const Geom& G, int i, int j) {
  if (!G.dxc) return G;
  Geom c = G;
  const double dx = G.dxc[i], dy = G.dyc[j];
  double lx = G.lxc[i], ly = G.lyc[j];
  const double mx = rmax(rmax(rmax(lx, ly), lx), ly), mn = rmin(rmin(rmin(lx, ly), lx), ly);
  if (mx - mn < 2.0 * 2.220446049250313080847263336181640625e-16) lx = ly = mx;
  c.l1 = lx; c.l2 = ly; c.l3 = lx; c.l4 = ly;
  c.vol = dx * dy - 0.0 * 0.0;
  c.dx = dx;
  c.dy = dy;
  c.inv_vol = 0.0;
  c.k1 = c.k2 = c.k3 = c.k4 = c.kinv = kNotPow2;
  return c;
}

// quad_cell_t metrics of a dx x dy axis-aligned cell (quad_cell.f90:69-229): volume dx*dy,
// edge lengths dx, dy, dx, dy (all set to the largest when they differ by < 2 eps),
// min_dx = dx, min_dy = dy.
inline Geom uniform_geom(double dx, double dy) {
  Geom G{};
  G.vol = (dx - 0.0) * (dy - 0.0) - (0.0 - 0.0) * (0.0 - 0.0);
  double l[4] = {dx, dy, dx, dy};
  double mx = l[0], mn = l[0];
  for (int k = 1; k < 4; ++k) { mx = l[k] > mx ? l[k] : mx; mn = l[k] < mn ? l[k] : mn; }
  if (mx - mn < 2.0 * 2.220446049250313080847263336181640625e-16) l[0] = l[1] = l[2] = l[3] = mx;
  G.l1 = l[0]; G.l2 = l[1]; G.l3 = l[2]; G.l4 = l[3];
  G.dx = dx;
  G.dy = dy;
  // a division by a power of two is the multiplication by its reciprocal, which is exactly
  // representable: both round the same real number (power-of-two grids, e.g. 4096^2 on [0,1]^2)
  int e = 0;
  const double m = std::frexp(G.vol, &e);
  G.inv_vol = (m == 0.5 && e > -1020 && e < 1020) ? 1.0 / G.vol : 0.0;
  auto pow2_exp = [](double x) {
    int ex = 0;
    const double mx = std::frexp(x, &ex);
    return (mx == 0.5 && ex > -1000 && ex < 1000) ? ex - 1 : kNotPow2;
  };
  G.k1 = pow2_exp(G.l1);
  G.k2 = pow2_exp(G.l2);
  G.k3 = pow2_exp(G.l3);
  G.k4 = pow2_exp(G.l4);
  G.kinv = G.inv_vol != 0.0 ? pow2_exp(G.inv_vol) : kNotPow2;
  return G;
}

// x * p for p = 2^k (k != kNotPow2): the exponent step when x and the product are normal, a
// signed zero for a zero x (p > 0); otherwise (and for any p that is not a power of two) the
// FP64 instruction; bit-identical to x * p
__device__ __forceinline__ double mul_pow2(double x, double p, int k) {
  const uint64_t u = intdiv::bits_of(x);
  const int e = (int)((u >> 52) & 0x7ffu);
  if (k != kNotPow2) {
    if ((u << 1) == 0ULL) return x;
    if (e >= 1 && e <= 2046 && e + k >= 1 && e + k <= 2046)
      return intdiv::double_of(u + ((uint64_t)(int64_t)k << 52));
  }
  return x * p;
}

__device__ __forceinline__ double divergence_fp64(double Fi, double Fim, double Fj, double Fjm,
                                                  const Geom& G) {
  const double REL_TOL = 1e-14;
  const double NEAR0 = 5.0 * Num<double>::tiny;  // near_zero, flux_solver.f90:461-474
  double mi = rmax(rmax(rabs(Fi), rabs(Fim)), 1.0);
  double mj = rmax(rmax(rabs(Fj), rabs(Fjm)), 1.0);
  // x / 1.0 is exact: skip the division when the scale is 1
  double a, b;
  // (the scale is 1 or above; compares on the integer pipe, mi * REL_TOL = REL_TOL for mi = 1)
  using N = Num<double>;
  const long long ONE = 0x3ff0000000000000LL;
  // products with the edge lengths: exponent steps when those are powers of two; x * 1.0 (the
  // scale is 1) is x itself
  if (__double_as_longlong(mi) == ONE) {
    a = mul_pow2(Fi, G.l2, G.k2) + (-mul_pow2(Fim, G.l4, G.k4));
    if (abs_lt(a, REL_TOL)) a = 0.0;
  } else {
    a = (mul_pow2(N::div(Fi, mi), G.l2, G.k2) + (-mul_pow2(N::div(Fim, mi), G.l4, G.k4))) * mi;
    if (abs_lt(a, mi * REL_TOL)) a = 0.0;
  }
  if (__double_as_longlong(mj) == ONE) {
    b = mul_pow2(Fj, G.l3, G.k3) + (-mul_pow2(Fjm, G.l1, G.k1));
    if (abs_lt(b, REL_TOL)) b = 0.0;
  } else {
    b = (mul_pow2(N::div(Fj, mj), G.l3, G.k3) + (-mul_pow2(N::div(Fjm, mj), G.l1, G.k1))) * mj;
    if (abs_lt(b, mj * REL_TOL)) b = 0.0;
  }
  double s = a + b;
  if (abs_lt(s, NEAR0)) s = 0.0;
  return G.inv_vol != 0.0 ? mul_pow2(-s, G.inv_vol, G.kinv) : N::div(-s, G.vol);
}

}  // namespace cato
