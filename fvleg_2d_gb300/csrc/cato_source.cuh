// cato_source.cuh -- the energy source term (source_t, src/lib/source_terms/mod_source.f90:63-425)
// as two small kernels per time step, ahead of the stage kernels that add the field to the
// energy residual (time_derivative, mod_fluid.f90:503).
//
// integrate (mod_source.f90:296-312), at the time t_n of the step start and on the density of
// U^n:
//   find_deposition_location: the critical density of the table at t_n (0 without a table: the
//     reference evaluates an interpolator that was never initialised, which returns zero), the
//     largest column i holding a density above it, x_center = that column's centroid (0 if none);
//   get_source_field: p_input = table(t_n) while t_n <= max_time (else 0), or the constant,
//     times the multiplier; then the geometry: uniform, constant_xy (with the reference's
//     centroid_x > ylo test), 1d_gaussian (constant in y) or decay.
// The column search is a max-reduction (atomicMax) into one of two slots; the field kernel
// reads this step's slot and resets the other for the next step.  exp and the real power of
// 'decay' are correctly rounded (dd_exp of cato_pbc.cuh); integer powers follow libgcc's
// __powidf2 square-and-multiply, which gfortran calls for x**n with a variable integer n.
#pragma once

#include "cato_ctl.cuh"
#include "cato_pbc.cuh"

namespace cato {

enum { SRC_UNIFORM = 0, SRC_CONSTANT_XY = 1, SRC_GAUSSIAN_1D = 2, SRC_DECAY = 3 };

struct SourceArgs {
  int geometry, order;
  int n;                      // table points (0: constant value)
  const double* t;            // table: time, source value, critical density
  const double* q;
  const double* rho_crit;
  double t_max;               // maxval(time) of the table
  double constant_value, multiplier;
  double xlo, xhi, ylo, yhi, fwhm_x;
  // grid: nodes (rectilinear) or uniform spacing from the origin
  const double* xn;
  const double* yn;
  double dx, dy;
  int ni, nj, pitch;
  const double* rho;          // density of U^n
  double* field;              // q_dot_h, one value per interior cell (pitch layout)
  int* i_dep;                 // two slots; this step uses slot `parity`
  int parity;
  const StepCtl* ctl;
};

__device__ __forceinline__ double exp_cr(double x) {
  if (!isfinite(x) || x > 709.0 || x < -745.0) return exp(x);
  if (x == 0.0) return 1.0;
  const ddouble e = dd_exp({x, 0.0});
  return e.hi + e.lo;
}

__device__ __forceinline__ double pow_cr(double x, double y) {
  if (!(x > 0.0) || !isfinite(x)) return pow(x, y);
  if (x == 1.0) return 1.0;
  return pow_dd(x, dd_log(x), y);
}

// x**n for integer n >= 0 (libgcc __powidf2)
__device__ __forceinline__ double powi(double x, int m) {
  unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

// linear_interp_1d%evaluate (finterp), as pbc_target
__device__ __forceinline__ double interp_table(int n, const double* xt, const double* f, double x) {
  int lo = 0, hi = n - 1;
  if (x >= xt[n - 1]) lo = n - 2;
  else if (x < xt[0]) lo = 0;
  else {
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (x < xt[mid]) hi = mid;
      else lo = mid;
    }
  }
  const double q1 = (x - xt[lo]) / (xt[lo + 1] - xt[lo]);
  const double p1 = 1.0 - q1;
  return p1 * f[lo] + q1 * f[lo + 1];
}

__device__ __forceinline__ double node_x(const SourceArgs& S, int i) {
  return S.xn ? S.xn[i] : (double)i * S.dx;
}
__device__ __forceinline__ double node_y(const SourceArgs& S, int j) {
  return S.yn ? S.yn[j] : (double)j * S.dy;
}
// quad_cell_t centroid (quad_cell.f90:145): ((x1 + x2) / 2, (y2 + y3) / 2) of the corners
__device__ __forceinline__ double centroid_x(const SourceArgs& S, int i) {
  return (node_x(S, i + 1) + node_x(S, i)) / 2.0;
}
__device__ __forceinline__ double centroid_y(const SourceArgs& S, int j) {
  return (node_y(S, j + 1) + node_y(S, j)) / 2.0;
}

// the largest column holding a density above the critical density
static __global__ void source_deposit_kernel(SourceArgs S) {
  if (!S.ctl->active) return;
  const double t = S.ctl->t_step;
  const double crit = S.n > 0 ? interp_table(S.n, S.t, S.rho_crit, t) : 0.0;
  int best = -1;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < (long long)S.ni * S.nj;
       c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % S.ni), j = (int)(c / S.ni);
    if (S.rho[(size_t)j * S.pitch + i] > crit && i > best) best = i;
  }
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_down_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best >= 0) atomicMax(S.i_dep + S.parity, best);
}

// q_dot_h of every interior cell
static __global__ void source_field_kernel(SourceArgs S) {
  const long long n0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (n0 == 0) S.i_dep[1 - S.parity] = -1;  // the next step's slot
  if (!S.ctl->active) return;
  const double t = S.ctl->t_step;
  double p_input;
  if (S.n == 0) p_input = S.constant_value;
  else p_input = t <= S.t_max ? interp_table(S.n, S.t, S.q, t) : 0.0;
  p_input = p_input * S.multiplier;
  const int id = S.i_dep[S.parity];
  const double x0 = id >= 0 ? centroid_x(S, id) : 0.0;
  for (long long c = n0; c < (long long)S.ni * S.nj; c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % S.ni), j = (int)(c / S.ni);
    double q = 0.0;
    if (fabs(p_input) > 0.0) {
      const double x = centroid_x(S, i);
      if (S.geometry == SRC_UNIFORM) {
        q = p_input;
      } else if (S.geometry == SRC_CONSTANT_XY) {
        const double y = centroid_y(S, j);
        if (x < S.xhi && x > S.xlo && y < S.yhi && x > S.ylo) q = p_input;
      } else if (S.geometry == SRC_GAUSSIAN_1D) {
        if (fabs(x - x0) < S.fwhm_x * 5.0) {
          const double d = x - x0;
          const double a = (d * d) / (2.0 * (S.fwhm_x * S.fwhm_x));
          q = p_input * exp_cr(-powi(a, S.order));
        }
      } else {  // decay
        if (x < x0) {
          q = p_input * exp_cr(-pow_cr(x / x0, 1.5)) / exp_cr(-1.0);
        } else {
          const double s = (x - x0) / x0;
          q = p_input * exp_cr(-(1e4 * (s * s)));
        }
      }
    }
    S.field[(size_t)j * S.pitch + i] = q;
  }
}

}  // namespace cato
