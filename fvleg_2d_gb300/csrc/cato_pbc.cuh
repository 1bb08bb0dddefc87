// cato_pbc.cuh -- the +x pressure-input boundary condition (pressure_input_bc.f90:256-414 with
// subsonic_outlet / subsonic_inlet of inlet_outlet.f90), evaluated once per stage for the
// boundary column before the stage kernel runs.
//
// Per stage: pbc_max_kernel takes the largest pressure of the last interior column (the
// reference's maxval over that column including its ghost rows, which hold copies of interior
// pressures), then pbc_edge_kernel computes the edge state (rho, u, p; v = 0) of every row
// -ng .. nj+ng-1 from the primitives of the last interior column of the same row.  The stage
// kernel reads that state for every +x ghost cell of the row.  The primitives come from the
// stage kernel's own loaders (load_src / src_to_prim), so they are the ones the stage sees.
//
// Exactness: the subsonic inlet raises to the real powers -gamma/(gamma-1) and -1/(gamma-1)
// (Fortran '**', i.e. libm pow).  pow_dd evaluates x**y in double-double arithmetic (Dekker's
// products and Knuth's sums, as in Hida, Li & Bailey's QD library) to about 2^-100 relative and
// rounds once, so it returns the correctly rounded power except when the exact value lies
// within ~2^-100 of a rounding midpoint.  A libm pow of < 1 ulp error returns the same double
// whenever it is correctly rounded.
#pragma once

#include "cato_ctl.cuh"
#include "cato_stage.cuh"

namespace cato {

// ---------------------------------------------------------------------------------------------
// double-double arithmetic (value = hi + lo, |lo| <= ulp(hi)/2)
// ---------------------------------------------------------------------------------------------
struct ddouble {
  double hi, lo;
};

__device__ __forceinline__ ddouble dd_quick_two_sum(double a, double b) {
  const double s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ ddouble dd_two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ ddouble dd_two_prod(double a, double b) {
  const double p = a * b;
  return {p, __fma_rn(a, b, -p)};
}
__device__ __forceinline__ ddouble dd_add(ddouble a, ddouble b) {
  ddouble s = dd_two_sum(a.hi, b.hi);
  const ddouble t = dd_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = dd_quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return dd_quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ddouble dd_add_d(ddouble a, double b) {
  ddouble s = dd_two_sum(a.hi, b);
  s.lo += a.lo;
  return dd_quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ddouble dd_mul(ddouble a, ddouble b) {
  ddouble p = dd_two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return dd_quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ ddouble dd_mul_d(ddouble a, double b) {
  ddouble p = dd_two_prod(a.hi, b);
  p.lo += a.lo * b;
  return dd_quick_two_sum(p.hi, p.lo);
}
// 1/n as a double-double (n a small integer, exact as a double)
__device__ __forceinline__ ddouble dd_recip(double n) {
  const double h = 1.0 / n;
  return {h, __fma_rn(-h, n, 1.0) / n};
}

// ln 2 = 0.693147180559945309417232121458176568075500134360255254120680...
__device__ __forceinline__ ddouble dd_ln2() {
  return {0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56};
}

// exp of a double-double argument of moderate size (|a| < 700): a = k ln2 + r, r = 2^10 s,
// expm1(s) by its Taylor series to s^9/9!, then expm1(2x) = expm1(x) (2 + expm1(x)) ten times.
__device__ inline ddouble dd_exp(ddouble a) {
  const double k = rint(a.hi / 0x1.62e42fefa39efp-1);
  ddouble r = dd_add(a, dd_mul_d(dd_ln2(), -k));
  r.hi = ldexp(r.hi, -10);
  r.lo = ldexp(r.lo, -10);
  // Horner: e = s (1 + s/2 (1 + s/3 (... (1 + s/9))))
  ddouble e = {1.0, 0.0};
#pragma unroll 1
  for (int n = 9; n >= 2; --n) {
    e = dd_mul(dd_mul(e, r), dd_recip((double)n));
    e = dd_add_d(e, 1.0);
  }
  e = dd_mul(e, r);
#pragma unroll 1
  for (int n = 0; n < 10; ++n) e = dd_mul(e, dd_add_d(e, 2.0));
  const ddouble y = dd_add_d(e, 1.0);
  const int ki = (int)k;
  return {ldexp(y.hi, ki), ldexp(y.lo, ki)};
}

// natural log of x > 0 as a double-double: one Newton step y + x exp(-y) - 1 from y = log(x)
// (quadratic convergence from the ~1 ulp start).
__device__ inline ddouble dd_log(double x) {
  const double y0 = log(x);
  const ddouble t = dd_mul_d(dd_exp({-y0, 0.0}), x);
  return dd_add_d(dd_add_d(t, -1.0), y0);
}

// x**y given lx = log(x) as a double-double, for finite x > 0 (the base of the isentropic
// relations is >= 1); anything else goes to libm's pow
__device__ __forceinline__ double pow_dd(double x, ddouble lx, double y) {
  if (!(x > 0.0) || !isfinite(x)) return pow(x, y);
  if (x == 1.0) return 1.0;
  const ddouble e = dd_exp(dd_mul_d(lx, y));
  return e.hi + e.lo;
}

// ---------------------------------------------------------------------------------------------
// the boundary state
// ---------------------------------------------------------------------------------------------
// subsonic_inlet (inlet_outlet.f90:60-165) for the +x boundary: normal (1, 0), domain v = 0,
// flow angle 0, inlet density rho_0 and total pressure p_0.  Operation order as written there.
__device__ inline void subsonic_inlet_px(double gamma, double rho, double u, double p,
                                         double rho_0, double p_0, double& rho_b, double& u_b,
                                         double& p_b) {
  const double v = 0.0, n_x = 1.0, n_y = 0.0;
  double cos_theta = 0.0;
  const double v_dot_n = u * (-n_x) + v * (-n_y);
  const double v_tot_d = sqrt(u * u + v * v);
  if (v_tot_d > 0.0) cos_theta = -v_dot_n / v_tot_d;
  const double cs_d = sqrt(gamma * p / rho);
  const double cs_0_sq = cs_d * cs_d + ((gamma - 1.0) / 2.0) * (v_tot_d * v_tot_d);
  const double R_minus = v_dot_n - (2.0 * cs_d / (gamma - 1.0));
  const double first =
      -(R_minus * (gamma - 1.0) / ((gamma - 1.0) * (cos_theta * cos_theta) + 2.0));
  double cs_b;
  if (fabs(cos_theta) > 0.0) {
    const double second = (((gamma - 1.0) * (cos_theta * cos_theta) + 2.0) * cs_0_sq) /
                          ((gamma - 1.0) * (R_minus * R_minus));
    const double third = (gamma - 1.0) / 2.0;
    cs_b = first * (1.0 + cos_theta * sqrt(second - third));
  } else {
    cs_b = first;
  }
  const double R_plus = v_dot_n + (2.0 * cs_b / (gamma - 1.0));
  const double v_tot_b = (2.0 * cs_b / (gamma - 1.0)) - R_plus;
  const double mach_b = v_tot_b / cs_b;
  u_b = v_tot_b * 1.0;  // cos(0)
  const double base = 1.0 + 0.5 * (gamma - 1.0) * (mach_b * mach_b);
  const bool use_log = base > 0.0 && isfinite(base) && base != 1.0;
  const ddouble lb = use_log ? dd_log(base) : ddouble{0.0, 0.0};
  p_b = p_0 * pow_dd(base, lb, -gamma / (gamma - 1.0));
  rho_b = rho_0 * pow_dd(base, lb, -1.0 / (gamma - 1.0));
}

// One row of apply_pressure_input_primitive_var_bc on +x (pressure_input_bc.f90:352-392):
// outflow (u > 0) subsonic, or supersonic while the boundary column's largest pressure is below
// the target: characteristic outlet at p_des (subsonic_outlet, inlet_outlet.f90:167-196);
// supersonic outflow: copy; supersonic inflow: (rho_des, u, p_des); subsonic inflow: inlet.
__device__ inline void pressure_input_edge(double gamma, double rho_d, double u_d, double p_d,
                                           double max_p, double p_des, double rho_des,
                                           double out[3]) {
  const double cs = sqrt(gamma * p_d / rho_d);
  const double mach_u = u_d / cs;
  double rb, ub, pb;
  if (mach_u > 0.0) {
    if (mach_u <= 1.0 || max_p < p_des) {
      pb = p_des;
      rb = rho_d + (pb - p_d) / (cs * cs);
      ub = u_d + 1.0 * (p_d - pb) / (rho_d * cs);
    } else {
      rb = rho_d;
      ub = u_d;
      pb = p_d;
    }
  } else if (fabs(mach_u) > 1.0) {
    rb = rho_des;
    ub = u_d;
    pb = p_des;
  } else {
    subsonic_inlet_px(gamma, rho_d, u_d, p_d, rho_des, p_des, rb, ub, pb);
  }
  out[0] = rb;
  out[1] = ub;
  out[2] = pb;
}

// Target pressure and density at time t: constants, or linear_interp_1d%evaluate of the table
// (finterp linear_interpolation_module.f90:730-762: the bracketing interval of dintrv, clamped to
// the first / last interval outside the table, then q = (t - t1)/(t2 - t1), (1 - q) f1 + q f2).
struct PbcTable {
  int n;                  // 0: constant target
  const double* t;        // n strictly increasing times
  const double* p;        // pressures at those times
  const double* rho;      // densities
  double p_const, rho_const;
};

__device__ inline void pbc_target(const PbcTable& T, double t, double& p, double& rho) {
  if (T.n == 0) {
    p = T.p_const;
    rho = T.rho_const;
    return;
  }
  int lo = 0, hi = T.n - 1;  // interval [lo, lo+1] with T.t[lo] <= t < T.t[lo+1]
  if (t >= T.t[T.n - 1]) {
    lo = T.n - 2;
  } else if (t < T.t[0]) {
    lo = 0;
  } else {
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (t < T.t[mid]) hi = mid;
      else lo = mid;
    }
  }
  const double q1 = (t - T.t[lo]) / (T.t[lo + 1] - T.t[lo]);
  const double p1 = 1.0 - q1;
  p = p1 * T.p[lo] + q1 * T.p[lo + 1];
  rho = p1 * T.rho[lo] + q1 * T.rho[lo + 1];
}

struct PbcArgs {
  PbcTable table;
  double* edge;        // (rho, u, p) of rows -ng .. nj+ng-1
  double* max_p;       // the column maximum of this stage
  const StepCtl* ctl;  // time and dt of the step
  int t_mode;          // 0: ctl->time (already t_n + dt); 1: ctl->t_create + ctl->dt
  int ng;
};

__device__ __forceinline__ double to_double(double x) { return x; }
__device__ __forceinline__ double to_double(float x) { return f2d_int(x); }
__device__ __forceinline__ double to_double(df x) { return from_df(x); }

// maxval as gfortran evaluates it: NaNs are skipped unless every element is NaN
__device__ __forceinline__ double max_skip_nan(double a, double b) {
  if (a != a) return b;
  if (b != b) return a;
  return b > a ? b : a;
}

// primitives (rho, u, v, p) of interior column sx, (possibly ghost) row `row`, as the stage
// kernel computes them
template <typename R>
__device__ __forceinline__ double prim_p_double(const StageArgs& A, int sx, int row, double q[4]) {
  RowSrc<R> s;
  load_src<R>(A, sx, row, s);
  R v[4];
  const R g = R(A.gamma), g1 = R(A.gamma - 1.0);
  src_to_prim<R>(A, s, false, 0, row, g, g1, v);
#pragma unroll
  for (int k = 0; k < 4; ++k) q[k] = to_double(v[k]);
  return q[3];
}

// the largest pressure of the last interior column (one CTA of 1024 threads)
template <typename R>
__global__ void __launch_bounds__(1024) pbc_max_kernel(StageArgs A, PbcArgs P) {
  __shared__ double red[32];
  double m = NAN;
  for (int j = threadIdx.x; j < A.nj; j += blockDim.x) {
    double q[4];
    m = max_skip_nan(m, prim_p_double<R>(A, A.ni - 1, j, q));
  }
  for (int o = 16; o > 0; o >>= 1) m = max_skip_nan(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : NAN;
    for (int o = 16; o > 0; o >>= 1) m = max_skip_nan(m, __shfl_down_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) *P.max_p = m;
  }
}

// the edge state of every row -ng .. nj+ng-1
template <typename R>
__global__ void pbc_edge_kernel(StageArgs A, PbcArgs P) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x - P.ng;
  if (r >= A.nj + P.ng) return;
  const double t = P.t_mode == 0 ? P.ctl->time : P.ctl->t_create + P.ctl->dt;
  double p_des, rho_des;
  pbc_target(P.table, t, p_des, rho_des);
  if (!(p_des >= Num<double>::tiny) || !(rho_des >= Num<double>::tiny)) {
    // get_desired_pressure / get_desired_density stop the reference here
    atomicOr(A.status, ST_BC_INPUT);
  }
  double q[4];
  prim_p_double<R>(A, A.ni - 1, r, q);
  double e[3];
  pressure_input_edge(A.gamma, q[0], q[1], q[3], *P.max_p, p_des, rho_des, e);
  double* o = P.edge + 3 * (size_t)(r + P.ng);
  o[0] = e[0];
  o[1] = e[1];
  o[2] = e[2];
}

// host: the two kernels of one stage on `s` (precision: enum cato_precision)
cudaError_t launch_pbc(int precision, const StageArgs& A, const PbcArgs& P, cudaStream_t s);

}  // namespace cato
