/*
 * cato_oracle.c -- TEST INFRASTRUCTURE ONLY: the parity oracle.
 *
 * A plain-C CPU restatement of the reference (smillerc/fvleg_2d, "CATO", Fortran 2018) FP64
 * time-step arithmetic for the hot path: primitive recovery, ghost-cell boundary conditions,
 * MUSCL TVD2 / MLP edge reconstruction, the AUSMPW+, SLAU family and Roe edge fluxes, the flux
 * divergence, the SSP-RK / rk(m,n) stage updates and the CFL time step.  Every function cites
 * the reference file:line it follows (paths relative to the reference repository root).
 * Operation order follows Fortran's left-to-right evaluation of each source expression, the
 * field operators' interior-only semantics and their epsilon flushes; build with
 * -ffp-contract=off so that no multiply-add is fused.
 *
 * AUSM+-up (driver), HLLC, the van Leer limiter and the Harten entropy fix have no runnable
 * reference code (see cato_gpu.h); their restatements here are marked "unpinned".
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this library; the
 * product (fvleg_2d_gb300/) never loads it.
 */
#include "cato_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* epsilon(1.0_rk), tiny(1.0_rk) */
#define EPS DBL_EPSILON
#define TINY DBL_MIN

static inline double dmax(double a, double b) { return (a < b) ? b : a; }
static inline double dmin(double a, double b) { return (b < a) ? b : a; }
/* Fortran SIGN(1.0, x): +1 for x >= +0, -1 for negative (incl. -0 in gfortran). */
static inline double fsign1(double x) { return signbit(x) ? -1.0 : 1.0; }

int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int oracle_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------------------------ */
/* indexing of halo-padded (1-ng:ni+ng, 1-ng:nj+ng) arrays                                     */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
  int ni, nj, ng, ld;
} dims_t;

static inline dims_t mkdims(const cato_config* c) {
  dims_t d = {c->ni, c->nj, c->n_ghost, c->ni + 2 * c->n_ghost};
  return d;
}
#define AT(a, i, j) (a)[((i) + d.ng - 1) + (size_t)((j) + d.ng - 1) * d.ld]
/* i-edge arrays (1:2, -1:ni, 0:nj) and j-edge arrays (1:2, 0:ni, -1:nj) */
#define IE(a, lr, i, j) (a)[(lr) + 2 * (((i) + 1) + (size_t)(j) * (d.ni + 2))]
#define JE(a, lr, i, j) (a)[(lr) + 2 * ((i) + (size_t)((j) + 1) * (d.ni + 1))]
/* edge flux arrays iflux(4, 0:ni, 1:nj) and jflux(4, 1:ni, 0:nj) */
#define IF(a, k, i, j) (a)[(k) + 4 * ((i) + (size_t)((j) - 1) * (d.ni + 1))]
#define JF(a, k, i, j) (a)[(k) + 4 * (((i) - 1) + (size_t)(j) * d.ni)]

static size_t nfield(dims_t d) { return (size_t)d.ld * (size_t)(d.nj + 2 * d.ng); }

/* ------------------------------------------------------------------------------------------ */
/* geometry: quad_cell_t (src/lib/geometry/quad_cell.f90:69-229) */
/* ------------------------------------------------------------------------------------------ */
void oracle_quad_metrics(const double xin[4], const double yin[4], double* volume,
                         double el[4], double nv[8], double* min_dx, double* min_dy) {
  double x[4], y[4];
  memcpy(x, xin, sizeof x);
  memcpy(y, yin, sizeof y);
  /* round-off snapping, quad_cell.f90:78-92 */
  if (fabs(y[1] - y[0]) < EPS) y[1] = y[0];
  if (fabs(y[3] - y[2]) < EPS) y[3] = y[2];
  if (fabs(x[2] - x[1]) < EPS) x[2] = x[1];
  if (fabs(x[3] - x[0]) < EPS) x[3] = x[0];
  /* calculate_volume, quad_cell.f90:176-191 */
  *volume = (x[1] - x[0]) * (y[3] - y[0]) - (x[3] - x[0]) * (y[1] - y[0]);
  /* calculate_edge_stats, quad_cell.f90:101-126 */
  el[0] = sqrt((x[1] - x[0]) * (x[1] - x[0]) + (y[1] - y[0]) * (y[1] - y[0]));
  el[1] = sqrt((x[2] - x[1]) * (x[2] - x[1]) + (y[2] - y[1]) * (y[2] - y[1]));
  el[2] = sqrt((x[3] - x[2]) * (x[3] - x[2]) + (y[3] - y[2]) * (y[3] - y[2]));
  el[3] = sqrt((x[0] - x[3]) * (x[0] - x[3]) + (y[0] - y[3]) * (y[0] - y[3]));
  double mx = dmax(dmax(dmax(el[0], el[1]), el[2]), el[3]);
  double mn = dmin(dmin(dmin(el[0], el[1]), el[2]), el[3]);
  if (mx - mn < 2.0 * EPS) el[0] = el[1] = el[2] = el[3] = mx;
  double midx[4], midy[4];
  midx[0] = (x[1] + x[0]) / 2.0; midy[0] = (y[1] + y[0]) / 2.0;
  midx[1] = (x[2] + x[1]) / 2.0; midy[1] = (y[2] + y[1]) / 2.0;
  midx[2] = (x[3] + x[2]) / 2.0; midy[2] = (y[3] + y[2]) / 2.0;
  midx[3] = (x[0] + x[3]) / 2.0; midy[3] = (y[0] + y[3]) / 2.0;
  *min_dx = dmin(fabs(x[1] - x[0]), fabs(x[2] - x[3]));
  *min_dy = dmin(fabs(y[3] - y[0]), fabs(y[2] - y[1]));
  /* calculate_edge_norm_vectors, quad_cell.f90:193-229 with vector.f90:68-96 */
  static const int head[4] = {1, 2, 3, 0};
  for (int e = 0; e < 4; ++e) {
    double ddx = x[head[e]] - midx[e];
    double ddy = y[head[e]] - midy[e];
    double vx = (midx[e] + ddy) - midx[e];
    double vy = (midy[e] - ddx) - midy[e];
    double len = sqrt(vx * vx + vy * vy);
    nv[2 * e] = vx / len;
    nv[2 * e + 1] = vy / len;
  }
}

/* Uniform Cartesian geometry shared by every cell: the quad_cell_t metrics of a dx x dy cell. */
typedef struct {
  double vol, l[4], dx, dy;
} geom_t;

static geom_t uniform_geom(const cato_config* c) {
  double x[4] = {0.0, c->dx, c->dx, 0.0}, y[4] = {0.0, 0.0, c->dy, c->dy};
  geom_t g;
  double nv[8];
  oracle_quad_metrics(x, y, &g.vol, g.l, nv, &g.dx, &g.dy);
  return g;
}

/* Per-cell metrics of a rectilinear grid with node coordinates x(1..ni+1), y(1..nj+1): the
 * quad_cell_t of every interior cell on its corners in the order of
 * grid_block_2d_t%populate_element_specifications (grid_block_2d.f90:370-387):
 * (x_i, y_j), (x_i+1, y_j), (x_i+1, y_j+1), (x_i, y_j+1).  Cell (i, j) is entry
 * (j-1)*ni + (i-1).  NULL on a bad grid (nodes not strictly increasing). */
static geom_t* rect_cells(int ni, int nj, const double* xn, const double* yn) {
  for (int i = 0; i < ni; ++i)
    if (!(xn[i + 1] > xn[i])) return NULL;
  for (int j = 0; j < nj; ++j)
    if (!(yn[j + 1] > yn[j])) return NULL;
  geom_t* g = (geom_t*)malloc(sizeof(geom_t) * (size_t)ni * nj);
  if (!g) return NULL;
  for (int j = 0; j < nj; ++j)
    for (int i = 0; i < ni; ++i) {
      double x[4] = {xn[i], xn[i + 1], xn[i + 1], xn[i]};
      double y[4] = {yn[j], yn[j], yn[j + 1], yn[j + 1]};
      double nv[8];
      geom_t* c = &g[(size_t)j * ni + i];
      oracle_quad_metrics(x, y, &c->vol, c->l, nv, &c->dx, &c->dy);
    }
  return g;
}

/* ------------------------------------------------------------------------------------------ */
/* limiters as inlined in muscl_tvd2.fypp:195-213                                              */
/* ------------------------------------------------------------------------------------------ */
double oracle_limiter(int32_t lim, double r) {
  switch (lim) {
    case CATO_LIM_MINMOD: return dmax(0.0, dmin(r, 1.0));
    case CATO_LIM_SUPERBEE: return dmax(dmax(0.0, dmin(2.0 * r, 1.0)), dmin(r, 2.0));
    case CATO_LIM_VAN_LEER: return (r + fabs(r)) / (1.0 + fabs(r)); /* unpinned: unreachable */
    default: return 0.0;
  }
}

/* ------------------------------------------------------------------------------------------ */
/* boundary conditions                                                                         */
/* ------------------------------------------------------------------------------------------ */
/* zero_gradient_bc.f90:64-119 (full-length rows/columns), symmetry_bc.f90:75-131,
 * periodic_bc.fypp:138-278 on a single image (x: rows jlo:jhi; y: columns ilo:ihi; corners
 * only when all four sides are periodic, periodic_bc.fypp:68-74). */
/* outlet_bc.f90:83-175: on +x every ghost column (all j of the halo) takes the characteristic
 * outflow state computed from the boundary column ihi; -x, +y, -y copy the boundary line
 * (full length). */
static void apply_outlet_px(dims_t d, double gamma, double p_b, double* f[4]) {
  const int ng = d.ng, ni = d.ni, nj = d.nj;
  double *rho = f[0], *u = f[1], *v = f[2], *p = f[3];
  for (int i = ni + 1; i <= ni + ng; ++i)
    for (int j = 1 - ng; j <= nj + ng; ++j) {
      double p_d = AT(p, ni, j), rho_0 = AT(rho, ni, j);
      if (p_b > TINY && rho_0 > TINY) {
        double cs = sqrt(gamma * fabs(p_d / rho_0));
        double vel = sqrt(AT(u, ni, j) * AT(u, ni, j) + AT(v, ni, j) * AT(v, ni, j));
        double mach = vel / cs;
        double nx = AT(u, ni, j) / (vel + 1e-30);
        double ny = AT(v, ni, j) / (vel + 1e-30);
        if (mach > 1.0) {
          AT(rho, i, j) = AT(rho, ni, j);
          AT(u, i, j) = AT(u, ni, j);
          AT(v, i, j) = AT(v, ni, j);
          AT(p, i, j) = AT(p, ni, j);
        } else {
          AT(rho, i, j) = AT(rho, ni, j) + (p_b - p_d) / (cs * cs);
          AT(u, i, j) = AT(u, ni, j) + nx * (p_d - p_b) / (rho_0 * cs);
          AT(v, i, j) = AT(v, ni, j) + ny * (p_d - p_b) / (rho_0 * cs);
          AT(p, i, j) = p_b;
        }
      }
    }
}

/* Target of a pressure-input side: a table in time (read_pressure_input, already scaled) or
 * the constants of the configuration; `time` is the boundary's time (its flux solver's). */
typedef struct {
  int n;
  const double *t, *p, *rho;
  double time;
} pbc_ctx_t;

/* linear_interp_1d%evaluate (finterp linear_interpolation_module.f90:730-762 with dintrv
 * :1189-1323): the interval [t(il), t(il+1)] holding x, the first / last interval outside. */
static double interp_1d(int n, const double* xt, const double* f, double x) {
  int il;
  if (x >= xt[n - 1]) il = n - 2;
  else if (x < xt[0]) il = 0;
  else {
    il = 0;
    while (il + 1 < n - 1 && xt[il + 1] <= x) ++il;
  }
  double q1 = (x - xt[il]) / (xt[il + 1] - xt[il]);
  double p1 = 1.0 - q1;
  return p1 * f[il] + q1 * f[il + 1];
}

/* Powers of the subsonic inlet.  The reference calls libm's pow (Fortran '**' on reals), which
 * is not always correctly rounded: glibc's pow has < 0.52 ulp of error, so an exact value very
 * close to a rounding midpoint can round the other way.  Mode 0 (default) calls pow as the
 * reference does; mode 1 returns the correctly rounded power from double-double arithmetic
 * (Dekker products via fma, Knuth sums; exp by a degree-9 Taylor series after k ln2 and 2^10
 * reductions, log by one Newton step on exp), the arithmetic the CUDA path uses. */
static int g_pow_mode = 0;

int oracle_set_pow_mode(int mode) {
  g_pow_mode = mode;
  return 0;
}

typedef struct {
  double hi, lo;
} ddo_t;

static ddo_t ddo_quick_two_sum(double a, double b) {
  double s = a + b;
  ddo_t r = {s, b - (s - a)};
  return r;
}
static ddo_t ddo_two_sum(double a, double b) {
  double s = a + b, bb = s - a;
  ddo_t r = {s, (a - (s - bb)) + (b - bb)};
  return r;
}
static ddo_t ddo_add(ddo_t a, ddo_t b) {
  ddo_t s = ddo_two_sum(a.hi, b.hi), t = ddo_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = ddo_quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return ddo_quick_two_sum(s.hi, s.lo);
}
static ddo_t ddo_add_d(ddo_t a, double b) {
  ddo_t s = ddo_two_sum(a.hi, b);
  s.lo += a.lo;
  return ddo_quick_two_sum(s.hi, s.lo);
}
static ddo_t ddo_mul(ddo_t a, ddo_t b) {
  double p = a.hi * b.hi;
  double e = fma(a.hi, b.hi, -p);
  e += a.hi * b.lo + a.lo * b.hi;
  return ddo_quick_two_sum(p, e);
}
static ddo_t ddo_mul_d(ddo_t a, double b) {
  double p = a.hi * b;
  double e = fma(a.hi, b, -p);
  e += a.lo * b;
  return ddo_quick_two_sum(p, e);
}
static ddo_t ddo_recip(double n) {
  double h = 1.0 / n;
  ddo_t r = {h, fma(-h, n, 1.0) / n};
  return r;
}
static ddo_t ddo_exp(ddo_t a) {
  const ddo_t ln2 = {0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56};
  double k = rint(a.hi / ln2.hi);
  ddo_t r = ddo_add(a, ddo_mul_d(ln2, -k));
  r.hi = ldexp(r.hi, -10);
  r.lo = ldexp(r.lo, -10);
  ddo_t e = {1.0, 0.0};
  for (int n = 9; n >= 2; --n) e = ddo_add_d(ddo_mul(ddo_mul(e, r), ddo_recip((double)n)), 1.0);
  e = ddo_mul(e, r);
  for (int n = 0; n < 10; ++n) e = ddo_mul(e, ddo_add_d(e, 2.0));
  ddo_t y = ddo_add_d(e, 1.0);
  ddo_t out = {ldexp(y.hi, (int)k), ldexp(y.lo, (int)k)};
  return out;
}
static double pow_cr(double x, double y) {
  if (!(x > 0.0) || !isfinite(x)) return pow(x, y);
  if (x == 1.0) return 1.0;
  double y0 = log(x);
  ddo_t m = {-y0, 0.0};
  ddo_t lx = ddo_add_d(ddo_add_d(ddo_mul_d(ddo_exp(m), x), -1.0), y0);
  ddo_t e = ddo_exp(ddo_mul_d(lx, y));
  return e.hi + e.lo;
}

double oracle_pow(int mode, double x, double y) { return mode ? pow_cr(x, y) : pow(x, y); }

static double exp_cr(double x) {
  if (!isfinite(x) || x > 709.0 || x < -745.0) return exp(x);
  if (x == 0.0) return 1.0;
  ddo_t a = {x, 0.0};
  ddo_t e = ddo_exp(a);
  return e.hi + e.lo;
}

static double bc_exp(double x) { return g_pow_mode ? exp_cr(x) : exp(x); }

/* x**n for a variable integer n (gfortran calls libgcc's __powidf2: square and multiply) */
static double powi(double x, int m) {
  unsigned n = m < 0 ? -(unsigned)m : (unsigned)m;
  double y = (n % 2) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2) y = y * x;
  }
  return m < 0 ? 1.0 / y : y;
}

static double bc_pow(double x, double y) { return g_pow_mode ? pow_cr(x, y) : pow(x, y); }

/* subsonic_inlet, inlet_outlet.f90:60-165, for the +x normal (1, 0), flow angle 0 */
static void subsonic_inlet(double gamma, const double dom[4], double inlet_density,
                           double inlet_total_press, double out[4]) {
  const double rho = dom[0], u = dom[1], v = dom[2], p = dom[3];
  const double n_x = 1.0, n_y = 0.0, theta = 0.0;
  double cos_theta = 0.0;
  double v_dot_n = u * (-n_x) + v * (-n_y);
  double v_tot_d = sqrt(u * u + v * v);
  if (v_tot_d > 0.0) cos_theta = -v_dot_n / v_tot_d;
  double cs_d = sqrt(gamma * p / rho);
  double cs_0_sq = cs_d * cs_d + ((gamma - 1.0) / 2.0) * (v_tot_d * v_tot_d);
  double R_minus = v_dot_n - (2.0 * cs_d / (gamma - 1.0));
  double first_term = -R_minus * (gamma - 1.0) / ((gamma - 1.0) * (cos_theta * cos_theta) + 2.0);
  double cs_b;
  if (fabs(cos_theta) > 0.0) {
    double second_term = (((gamma - 1.0) * (cos_theta * cos_theta) + 2.0) * cs_0_sq) /
                         ((gamma - 1.0) * (R_minus * R_minus));
    double third_term = (gamma - 1.0) / 2.0;
    cs_b = first_term * (1.0 + cos_theta * sqrt(second_term - third_term));
  } else {
    cs_b = first_term;
  }
  double R_plus = v_dot_n + (2.0 * cs_b / (gamma - 1.0));
  double v_tot_b = (2.0 * cs_b / (gamma - 1.0)) - R_plus;
  double mach_b = v_tot_b / cs_b;
  double u_b = v_tot_b * cos(theta);
  double v_b = v_tot_b * sin(theta);
  double p_b = inlet_total_press *
               bc_pow(1.0 + 0.5 * (gamma - 1.0) * (mach_b * mach_b), -gamma / (gamma - 1.0));
  double rho_b = inlet_density *
                 bc_pow(1.0 + 0.5 * (gamma - 1.0) * (mach_b * mach_b), -1.0 / (gamma - 1.0));
  out[0] = rho_b; out[1] = u_b; out[2] = v_b; out[3] = p_b;
}

/* apply_pressure_input_primitive_var_bc on +x, pressure_input_bc.f90:256-404: edge states of
 * every row bottom_ghost..top_ghost from the boundary column ihi, then every ghost column. */
static void apply_pressure_input_px(dims_t d, double gamma, double p_const, double rho_const,
                                    const pbc_ctx_t* pc, double* f[4]) {
  const int ng = d.ng, ni = d.ni, nj = d.nj, nrow = nj + 2 * ng;
  double *rho = f[0], *u = f[1], *v = f[2], *p = f[3];
  double p_des = p_const, rho_des = rho_const;
  if (pc && pc->n > 0) {
    p_des = interp_1d(pc->n, pc->t, pc->p, pc->time);
    rho_des = interp_1d(pc->n, pc->t, pc->rho, pc->time);
  }
  double* edge = (double*)malloc(sizeof(double) * 3 * (size_t)nrow);
  /* maxval(domain_p(bottom:top)): gfortran skips NaNs unless all are NaN */
  double maxp = NAN;
  for (int j = 1 - ng; j <= nj + ng; ++j) {
    double x = AT(p, ni, j);
    if (maxp != maxp || x > maxp) maxp = (x != x) ? maxp : x;
  }
  for (int j = 1 - ng; j <= nj + ng; ++j) {
    double dom[4] = {AT(rho, ni, j), AT(u, ni, j), 0.0, AT(p, ni, j)};
    double b[4];
    double cs = sqrt(gamma * dom[3] / dom[0]);
    double mach_u = dom[1] / cs;
    if (mach_u > 0.0) {
      if (mach_u <= 1.0 || maxp < p_des) {
        /* subsonic_outlet, inlet_outlet.f90:167-196 with the normal (1, 0) */
        double cs_d = sqrt(gamma * dom[3] / dom[0]);
        b[3] = p_des;
        b[0] = dom[0] + (b[3] - dom[3]) / (cs_d * cs_d);
        b[1] = dom[1] + 1.0 * (dom[3] - b[3]) / (dom[0] * cs_d);
        b[2] = dom[2] + 0.0 * (dom[3] - b[3]) / (dom[0] * cs_d);
      } else {
        for (int k = 0; k < 4; ++k) b[k] = dom[k]; /* supersonic_outlet */
      }
    } else {
      if (fabs(mach_u) > 1.0) {
        b[0] = rho_des; b[1] = dom[1]; b[2] = dom[2]; b[3] = p_des;
      } else {
        subsonic_inlet(gamma, dom, rho_des, p_des, b);
      }
    }
    double* e = edge + 3 * (size_t)(j + ng - 1);
    e[0] = b[0]; e[1] = b[1]; e[2] = b[3];
  }
  for (int i = ni + 1; i <= ni + ng; ++i)
    for (int j = 1 - ng; j <= nj + ng; ++j) {
      const double* e = edge + 3 * (size_t)(j + ng - 1);
      AT(rho, i, j) = e[0];
      AT(u, i, j) = e[1];
      AT(v, i, j) = 0.0;
      AT(p, i, j) = e[2];
    }
  free(edge);
}

/* jlo..jhi: the rows the x-periodic copy covers: the interior rows (periodic_bc.fypp:176-192),
 * and the ghost rows beyond a slab's exchange side, which are interior rows of the whole grid */
static void apply_one_bc(dims_t d, int type, int side, int do_corners, double gamma,
                         double p_b, double rho_b, const pbc_ctx_t* pc, double* f[4], int jlo,
                         int jhi) {
  const int ng = d.ng, ni = d.ni, nj = d.nj;
  if (type == CATO_BC_EXCHANGE) return; /* filled from the neighbouring slab */
  if (type == CATO_BC_PRESSURE_INPUT) {
    if (side == CATO_PLUS_X) apply_pressure_input_px(d, gamma, p_b, rho_b, pc, f);
    return;
  }
  if (type == CATO_BC_OUTLET) {
    if (side == CATO_PLUS_X) {
      apply_outlet_px(d, gamma, p_b, f);
      return;
    }
    type = CATO_BC_ZERO_GRADIENT; /* the line copies of outlet_bc.f90:126-164 */
  }
  for (int g = 1; g <= ng; ++g) {
    if (type == CATO_BC_ZERO_GRADIENT) {
      for (int k = 0; k < 4; ++k) {
        double* a = f[k];
        if (side == CATO_PLUS_X)
          for (int j = 1 - ng; j <= nj + ng; ++j) AT(a, ni + g, j) = AT(a, ni, j);
        if (side == CATO_MINUS_X)
          for (int j = 1 - ng; j <= nj + ng; ++j) AT(a, 1 - g, j) = AT(a, 1, j);
        if (side == CATO_PLUS_Y)
          for (int i = 1 - ng; i <= ni + ng; ++i) AT(a, i, nj + g) = AT(a, i, nj);
        if (side == CATO_MINUS_Y)
          for (int i = 1 - ng; i <= ni + ng; ++i) AT(a, i, 1 - g) = AT(a, i, 1);
      }
    } else if (type == CATO_BC_SYMMETRY) {
      for (int k = 0; k < 4; ++k) {
        double* a = f[k];
        /* normal velocity negated: u (k=1) on +-x, v (k=2) on +-y */
        int neg_x = (k == 1), neg_y = (k == 2);
        if (side == CATO_PLUS_X)
          for (int j = 1 - ng; j <= nj + ng; ++j)
            AT(a, ni + g, j) = neg_x ? -AT(a, ni - (g - 1), j) : AT(a, ni - (g - 1), j);
        if (side == CATO_MINUS_X)
          for (int j = 1 - ng; j <= nj + ng; ++j)
            AT(a, 1 - g, j) = neg_x ? -AT(a, 1 + (g - 1), j) : AT(a, 1 + (g - 1), j);
        if (side == CATO_PLUS_Y)
          for (int i = 1 - ng; i <= ni + ng; ++i)
            AT(a, i, nj + g) = neg_y ? -AT(a, i, nj - (g - 1)) : AT(a, i, nj - (g - 1));
        if (side == CATO_MINUS_Y)
          for (int i = 1 - ng; i <= ni + ng; ++i)
            AT(a, i, 1 - g) = neg_y ? -AT(a, i, 1 + (g - 1)) : AT(a, i, 1 + (g - 1));
      }
    }
  }
  if (type == CATO_BC_PERIODIC) {
    for (int k = 0; k < 4; ++k) {
      double* a = f[k];
      if (side == CATO_PLUS_X || side == CATO_MINUS_X) {
        /* ihi+1:ihi_halo <- ilo:ilo+ng-1 ; ilo_halo:ilo-1 <- ihi-ng+1:ihi */
        for (int j = jlo; j <= jhi; ++j)
          for (int g = 1; g <= ng; ++g) {
            AT(a, ni + g, j) = AT(a, g, j);
            AT(a, 1 - g, j) = AT(a, ni + 1 - g, j);
          }
      } else {
        for (int i = 1; i <= ni; ++i)
          for (int g = 1; g <= ng; ++g) {
            AT(a, i, nj + g) = AT(a, i, g);
            AT(a, i, 1 - g) = AT(a, i, nj + 1 - g);
          }
      }
      if (do_corners) {
        for (int gi = 1; gi <= ng; ++gi)
          for (int gj = 1; gj <= ng; ++gj) {
            AT(a, 1 - gi, 1 - gj) = AT(a, ni + 1 - gi, nj + 1 - gj);
            AT(a, ni + gi, 1 - gj) = AT(a, gi, nj + 1 - gj);
            AT(a, 1 - gi, nj + gj) = AT(a, ni + 1 - gi, gj);
            AT(a, ni + gi, nj + gj) = AT(a, gi, gj);
          }
      }
    }
  }
}

/* periodic 2, zero-gradient / symmetry 1, outlet and pressure input 0 (the constructors); a
 * slab's exchange side is no boundary condition (-1: never applied) */
static int bc_priority(int type) {
  if (type == CATO_BC_EXCHANGE) return -1;
  return type == CATO_BC_PERIODIC ? 2
         : (type == CATO_BC_OUTLET || type == CATO_BC_PRESSURE_INPUT ? 0 : 1);
}

/* flux_solver_t%apply_primitive_bc, flux_solver.f90:138-185: priority high -> low and, within
 * one priority, +x, +y, -x, -y. */
static int apply_bc_at(const cato_config* c, const pbc_ctx_t* pc, double* rho, double* u,
                       double* v, double* p) {
  dims_t d = mkdims(c);
  double* f[4] = {rho, u, v, p};
  int all_periodic = 1;
  for (int s = 0; s < 4; ++s) all_periodic &= (c->bc[s] == CATO_BC_PERIODIC);
  int maxp = 0;
  for (int s = 0; s < 4; ++s) maxp = bc_priority(c->bc[s]) > maxp ? bc_priority(c->bc[s]) : maxp;
  const int jlo = c->bc[CATO_MINUS_Y] == CATO_BC_EXCHANGE ? 1 - d.ng : 1;
  const int jhi = c->bc[CATO_PLUS_Y] == CATO_BC_EXCHANGE ? d.nj + d.ng : d.nj;
  for (int prio = maxp; prio >= 0; --prio)
    for (int s = 0; s < 4; ++s)
      if (bc_priority(c->bc[s]) == prio)
        apply_one_bc(d, c->bc[s], s, all_periodic, c->gamma, c->bc_pressure, c->bc_density,
                     pc, f, jlo, jhi);
  return 0;
}

int oracle_apply_bc(const cato_config* c, double* rho, double* u, double* v, double* p) {
  return apply_bc_at(c, NULL, rho, u, v, p);
}

/* One boundary_condition_t%apply on one side (used to replay the reference's own BC unit tests,
 * tests/unit/test_bc/mod_test_bc.f90, which apply single sides). */
int oracle_apply_bc_side(const cato_config* c, int side, int type, int do_corners, double* rho,
                         double* u, double* v, double* p) {
  dims_t d = mkdims(c);
  double* f[4] = {rho, u, v, p};
  apply_one_bc(d, type, side, do_corners, c->gamma, c->bc_pressure, c->bc_density, NULL, f, 1,
               d.nj);
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* reconstruction                                                                              */
/* ------------------------------------------------------------------------------------------ */
/* cell value along the edge-normal direction: offset n along the normal, t along the tangent */
#define QN(n, t) (dir == 0 ? AT(q, i + (n), j + (t)) : AT(q, i + (t), j + (n)))

/* muscl_tvd2.fypp:172-223 for one edge (i,j) in direction dir (0 = i, 1 = j). */
static void tvd2_edge(dims_t d, int lim, const double* q, int dir, int i, int j, double* L,
                      double* R) {
  double dm = QN(0, 0) - QN(-1, 0);
  double d0 = QN(1, 0) - QN(0, 0);
  double dp = QN(2, 0) - QN(1, 0);
  if (fabs(dm) < EPS) dm = 0.0;
  if (fabs(d0) < EPS) d0 = 0.0;
  if (fabs(dp) < EPS) dp = 0.0;
  double rL = d0 / (dm + 1e-16);
  double rR = d0 / (dp + 1e-16);
  double phi = oracle_limiter(lim, rL);
  *L = QN(0, 0) + 0.5 * phi * dm;
  phi = oracle_limiter(lim, rR);
  *R = QN(1, 0) - 0.5 * phi * dp;
}

/* muscl_mlp.fypp:190-281 (Kim & Kim 2005 MLP) for one edge; order 3 or 5. */
static void mlp_edge(dims_t d, int order, const double* q, int dir, int i, int j, double* L,
                     double* R) {
  const double S = 1e-30; /* SMALL_NUM, muscl_mlp.fypp:122 */
  double dm = QN(0, 0) - QN(-1, 0);
  double d0 = QN(1, 0) - QN(0, 0);
  double dp = QN(2, 0) - QN(1, 0);
  if (fabs(dm) < EPS) dm = 0.0;
  if (fabs(d0) < EPS) d0 = 0.0;
  if (fabs(dp) < EPS) dp = 0.0;
  double dm3 = 0.0, dp5 = 0.0;
  if (order == 5) {
    dm3 = QN(-1, 0) - QN(-2, 0);
    dp5 = QN(3, 0) - QN(2, 0);
    if (fabs(dm3) < EPS) dm3 = 0.0;
    if (fabs(dp5) < EPS) dp5 = 0.0;
  }
  double rR_p1 = d0 / (dp + S);
  double rL = d0 / (dm + S);
  double bL, bR;
  if (order == 5) {
    double rL_m1 = dm / (dm3 + S);
    double rL_p1 = dp / (d0 + S);
    double rR_p2 = dp / (dp5 + S);
    double rR = dm / (d0 + S);
    bL = ((((-2.0 / (rL_m1 + S)) + 11.0) + 24.0 * rL) - 3.0 * rL * rL_p1) / 30.0;
    bR = ((((-2.0 / (rR_p2 + S)) + 11.0) + 24.0 * rR_p1) - 3.0 * rR_p1 * rR) / 30.0;
  } else {
    bL = (1.0 + 2.0 * rL) / 3.0;
    bR = (1.0 + 2.0 * rR_p1) / 3.0;
  }
  /* tan(theta) with the transverse neighbours, muscl_mlp.fypp:241-249 */
  double tt = fabs(QN(0, 1) - QN(0, -1)) / (fabs(QN(1, 0) - QN(-1, 0)) + S);
  double tt1 = fabs(QN(1, 1) - QN(1, -1)) / (fabs(QN(2, 0) - QN(0, 0)) + S);
  double aLt = (2.0 * dmax(1.0, rL) * (1.0 + dmax(0.0, tt1 / (rR_p1 + S)))) / (1.0 + tt);
  double aRt = (2.0 * dmax(1.0, rR_p1) * (1.0 + dmax(0.0, tt / (rL + S)))) / (1.0 + tt1);
  double aL = dmax(1.0, dmin(2.0, aLt));
  double aR = dmax(1.0, dmin(2.0, aRt));
  *L = QN(0, 0) + 0.5 * dmax(0.0, dmin(dmin(aL * rL, aL), bL)) * dm;
  *R = QN(1, 0) - 0.5 * dmax(0.0, dmin(dmin(aR * rR_p1, aR), bR)) * dp;
}
#undef QN

static void edge_recon(dims_t d, int lim, const double* q, int dir, int i, int j, double* L,
                       double* R) {
  if (lim == CATO_LIM_MLP3) mlp_edge(d, 3, q, dir, i, j, L, R);
  else if (lim == CATO_LIM_MLP5) mlp_edge(d, 5, q, dir, i, j, L, R);
  else tvd2_edge(d, lim, q, dir, i, j, L, R);
}

/* muscl_interpolation_t%interpolate_edge_values (muscl_tvd2.fypp:126-227, muscl_mlp.fypp:
 * 117-284): i-edges (L/R, -1:ni, 0:nj) computed for i = 0..ni, j = 0..nj (the i = -1 slot stays
 * 0); j-edges (L/R, 0:ni, -1:nj) for i = 0..ni, j = 0..nj. */
int oracle_interpolate_edges(const cato_config* c, const double* q, double* ie, double* je) {
  dims_t d = mkdims(c);
  memset(ie, 0, sizeof(double) * 2 * (size_t)(d.ni + 2) * (d.nj + 1));
  memset(je, 0, sizeof(double) * 2 * (size_t)(d.ni + 1) * (d.nj + 2));
#pragma omp parallel for schedule(static)
  for (int j = 0; j <= d.nj; ++j)
    for (int i = 0; i <= d.ni; ++i) {
      edge_recon(d, c->limiter, q, 0, i, j, &IE(ie, 0, i, j), &IE(ie, 1, i, j));
      edge_recon(d, c->limiter, q, 1, i, j, &JE(je, 0, i, j), &JE(je, 1, i, j));
    }
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* edge fluxes                                                                                 */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
  double r, u, v, p;
} prim_t;

/* AUSMPW+ split functions, ausmpw_plus_solver.fypp:486-530 (alpha = 1/8, :61) */
static double ausmpw_p_plus(double M) {
  const double alpha = 1.0 / 8.0;
  if (fabs(M) > 1.0) return 0.5 * (1.0 + fsign1(M));
  return 0.25 * ((M + 1.0) * (M + 1.0)) * (2.0 - M) + alpha * M * ((M * M - 1.0) * (M * M - 1.0));
}
static double ausmpw_p_minus(double M) {
  const double alpha = 1.0 / 8.0;
  if (fabs(M) > 1.0) return 0.5 * (1.0 - fsign1(M));
  return 0.25 * ((M - 1.0) * (M - 1.0)) * (2.0 + M) - alpha * M * ((M * M - 1.0) * (M * M - 1.0));
}
static double ausmpw_m_plus(double M) {
  if (fabs(M) > 1.0) return 0.5 * (M + fabs(M));
  return 0.25 * ((M + 1.0) * (M + 1.0));
}
static double ausmpw_m_minus(double M) {
  if (fabs(M) > 1.0) return 0.5 * (M - fabs(M));
  return -(0.25 * ((M - 1.0) * (M - 1.0)));
}

/* AUSMPW+ edge flux, ausmpw_plus_solver.fypp:336-459 with get_f (:532-556) and get_w
 * (:558-568).  pc = cell pressures p1_L, p1_R, p2_L, p2_R. */
static void flux_ausmpw(const cato_config* c, int dir, double nx, double ny, prim_t Lq, prim_t Rq,
                        const double pc[4], double F[4]) {
  const double g = c->gamma;
  double rho_L = Lq.r, u_LHS = Lq.u, v_LHS = Lq.v, p_L = Lq.p;
  double rho_R = Rq.r, u_RHS = Rq.u, v_RHS = Rq.v, p_R = Rq.p;
  double U_L, U_R, V_L, V_R;
  if (dir == 0) { U_L = u_LHS; U_R = u_RHS; V_L = v_LHS; V_R = v_RHS; }
  else { U_L = v_LHS; U_R = v_RHS; V_L = u_LHS; V_R = u_RHS; }
  double cs_L = sqrt(g * p_L / rho_L);
  double cs_R = sqrt(g * p_R / rho_R);
  double M_LHS = sqrt(u_LHS * u_LHS + v_LHS * v_LHS) / cs_L;
  double M_RHS = sqrt(u_RHS * u_RHS + v_RHS * v_RHS) / cs_R;
  if (c->apply_low_mach_fix && (fabs(M_LHS) < 0.1 || fabs(M_RHS) < 0.1)) { /* LOW_MACH */
    double f_M = dmin(1.0, dmax(M_LHS, M_RHS));
    double uLf = 0.5 * (u_LHS + u_RHS) + f_M * 0.5 * (u_LHS - u_RHS);
    double uRf = 0.5 * (u_LHS + u_RHS) - f_M * 0.5 * (u_LHS - u_RHS);
    double vLf = 0.5 * (v_LHS + v_RHS) + f_M * 0.5 * (v_LHS - v_RHS);
    double vRf = 0.5 * (v_LHS + v_RHS) - f_M * 0.5 * (v_LHS - v_RHS);
    u_LHS = uLf; u_RHS = uRf; v_LHS = vLf; v_RHS = vRf;
  }
  double H_L = (g / (g - 1.0)) * (p_L / rho_L) + 0.5 * (u_LHS * u_LHS + v_LHS * v_LHS);
  double H_R = (g / (g - 1.0)) * (p_R / rho_R) + 0.5 * (u_RHS * u_RHS + v_RHS * v_RHS);
  double H_normal = dmin(H_L - 0.5 * (V_L * V_L), H_R - 0.5 * (V_R * V_R));
  double c_s = sqrt(2.0 * ((g - 1.0) / (g + 1.0)) * H_normal);
  double c_half;
  if (0.5 * (U_L + U_R) < 0.0) c_half = (c_s * c_s) / dmax(fabs(U_R), c_s);
  else c_half = (c_s * c_s) / dmax(fabs(U_L), c_s);
  double M_L = U_L / c_half;
  double M_R = U_R / c_half;
  double M_L_plus = ausmpw_m_plus(M_L);
  double M_R_minus = ausmpw_m_minus(M_R);
  double P_R_minus = ausmpw_p_minus(M_R);
  double P_L_plus = ausmpw_p_plus(M_L);
  double p_s = p_L * P_L_plus + p_R * P_R_minus;
  double mt = dmin(p_L / p_R, p_R / p_L);
  double w = 1.0 - mt * mt * mt;
  double f_L, f_R;
  if (fabs(p_s) < TINY) {
    f_L = 0.0;
    f_R = 0.0;
  } else {
    double t = dmin(1.0, dmin(dmin(dmin(pc[0], pc[1]), pc[2]), pc[3]) / dmin(p_L, p_R));
    double min_term = t * t;
    f_L = ((p_L / p_s) - 1.0) * min_term;
    f_R = ((p_R / p_s) - 1.0) * min_term;
  }
  double Mb_L, Mb_R;
  if (M_L_plus + M_R_minus < 0.0) {
    Mb_L = M_L_plus * w * (1.0 + f_L);
    Mb_R = M_R_minus + M_L_plus * ((1.0 - w) * (1.0 + f_L) - f_R);
  } else {
    Mb_L = M_L_plus + M_R_minus * ((1.0 - w) * (1.0 + f_R) - f_L);
    Mb_R = M_R_minus * w * (1.0 + f_R);
  }
  double mL = Mb_L * c_half * rho_L;
  double mR = Mb_R * c_half * rho_R;
  F[0] = mL + mR;
  F[1] = (mL * u_LHS) + (mR * u_RHS) + ((P_L_plus * nx * p_L) + (P_R_minus * nx * p_R));
  F[2] = (mL * v_LHS) + (mR * v_RHS) + ((P_L_plus * ny * p_L) + (P_R_minus * ny * p_R));
  F[3] = (mL * H_L) + (mR * H_R);
}

/* M-AUSMPW+ (m_ausmpw_plus_solver.fypp, the active code of get_iflux/get_jflux :437-708): the
 * AUSMPW+ interface Mach and pressure splitting without the alpha term (:600-610), the shock
 * sensor f of get_f (:804-843, 1e-10 cuts), and interface states blended towards the superbee
 * states by phi_L_half / phi_R_half (:768-800); flux cuts at epsilon*1e3 (:369, :684-705). */
static double mausm_p_plus(double M) {
  if (fabs(M) > 1.0) return 0.5 * (1.0 + (signbit(M) ? -1.0 : 1.0));
  return 0.25 * ((M + 1.0) * (M + 1.0)) * (2.0 - M);
}
static double mausm_p_minus(double M) {
  if (fabs(M) > 1.0) return 0.5 * (1.0 - (signbit(M) ? -1.0 : 1.0));
  return 0.25 * ((M - 1.0) * (M - 1.0)) * (2.0 + M);
}
static double mausm_phi_L(double pL, double pR, double pLsb, double a) {
  if (fabs(pR - pL) < 1.0 || fabs(pLsb - pL) < EPS) return pL;
  return pL + dmax(0.0, (pR - pL) * (pLsb - pL)) / ((pR - pL) * fabs(pLsb - pL)) *
                  dmin(dmin(a, 0.5 * fabs(pR - pL)), fabs(pLsb - pL));
}
static double mausm_phi_R(double pL, double pR, double pRsb, double a) {
  if (fabs(pL - pR) < EPS || fabs(pRsb - pR) < 1.0) return pR;
  return pR + dmax(0.0, (pL - pR) * (pRsb - pR)) / ((pL - pR) * fabs(pRsb - pR)) *
                  dmin(dmin(a, 0.5 * fabs(pL - pR)), fabs(pRsb - pR));
}
static void flux_mausmpw(const cato_config* c, int dir, double nx, double ny, prim_t Lq,
                         prim_t Rq, prim_t Ls, prim_t Rs, const double pc[4], double F[4]) {
  const double g = c->gamma;
  const double EPSF = EPS * 1e3; /* epsilon(1.0_rk) * 1e3_rk */
  double rho_L = Lq.r, u_LHS = Lq.u, v_LHS = Lq.v, p_L = Lq.p;
  double rho_R = Rq.r, u_RHS = Rq.u, v_RHS = Rq.v, p_R = Rq.p;
  double U_L, U_R, V_L, V_R; /* taken before the low-Mach fix */
  if (dir == 0) { U_L = u_LHS; U_R = u_RHS; V_L = v_LHS; V_R = v_RHS; }
  else { U_L = v_LHS; U_R = v_RHS; V_L = u_LHS; V_R = u_RHS; }
  double cs_L = sqrt(g * p_L / rho_L);
  double cs_R = sqrt(g * p_R / rho_R);
  double M_LHS = sqrt(u_LHS * u_LHS + v_LHS * v_LHS) / cs_L;
  double M_RHS = sqrt(u_RHS * u_RHS + v_RHS * v_RHS) / cs_R;
  if (c->apply_low_mach_fix && (fabs(M_LHS) < 0.1 || fabs(M_RHS) < 0.1)) { /* LOW_MACH */
    double f_M = dmin(1.0, dmax(M_LHS, M_RHS));
    double uLf = 0.5 * (u_LHS + u_RHS) + f_M * 0.5 * (u_LHS - u_RHS);
    double uRf = 0.5 * (u_LHS + u_RHS) - f_M * 0.5 * (u_LHS - u_RHS);
    double vLf = 0.5 * (v_LHS + v_RHS) + f_M * 0.5 * (v_LHS - v_RHS);
    double vRf = 0.5 * (v_LHS + v_RHS) - f_M * 0.5 * (v_LHS - v_RHS);
    u_LHS = uLf; u_RHS = uRf; v_LHS = vLf; v_RHS = vRf;
  }
  double H_L = (g / (g - 1.0)) * (p_L / rho_L) + 0.5 * (u_LHS * u_LHS + v_LHS * v_LHS);
  double H_R = (g / (g - 1.0)) * (p_R / rho_R) + 0.5 * (u_RHS * u_RHS + v_RHS * v_RHS);
  double H_normal = dmin(H_L - 0.5 * (V_L * V_L), H_R - 0.5 * (V_R * V_R));
  double c_s = sqrt(2.0 * ((g - 1.0) / (g + 1.0)) * H_normal);
  double c_half;
  if (0.5 * (U_L + U_R) < 0.0) c_half = (c_s * c_s) / dmax(fabs(U_R), c_s);
  else c_half = (c_s * c_s) / dmax(fabs(U_L), c_s);
  double M_L = U_L / c_half;
  double M_R = U_R / c_half;
  double M_L_plus = ausmpw_m_plus(M_L);
  double M_R_minus = ausmpw_m_minus(M_R);
  double P_R_minus = mausm_p_minus(M_R);
  double P_L_plus = mausm_p_plus(M_L);
  double p_s = p_L * P_L_plus + p_R * P_R_minus;
  double mt = dmin(p_L / p_R, p_R / p_L);
  double w = 1.0 - (mt * mt * mt);
  double f_L, f_R;
  if (fabs(p_s) < TINY) {
    f_L = 0.0;
    f_R = 0.0;
  } else {
    double t = dmin(1.0, dmin(dmin(dmin(pc[0], pc[1]), pc[2]), pc[3]) / dmin(p_L, p_R));
    double min_term = t * t;
    if (fabs(1.0 - min_term) < 1e-10) min_term = 1.0;
    double fl = (p_L / p_s) - 1.0;
    if (fabs(fl) < 1e-10) fl = 0.0;
    f_L = fl * min_term;
    double fr = (p_R / p_s) - 1.0;
    if (fabs(fr) < 1e-10) fr = 0.0;
    f_R = fr * min_term;
  }
  double Mb_L, Mb_R;
  if (M_L_plus + M_R_minus < 0.0) {
    Mb_L = M_L_plus * w * (1.0 + f_L);
    Mb_R = M_R_minus + M_L_plus * ((1.0 - w) * (1.0 + f_L) - f_R);
  } else {
    Mb_L = M_L_plus + M_R_minus * ((1.0 - w) * (1.0 + f_R) - f_L);
    Mb_R = M_R_minus * w * (1.0 + f_R);
  }
  double t2 = dmin(1.0, dmax(fabs(M_L), fabs(M_R)));
  double a = 1.0 - t2 * t2;
  double rLh = mausm_phi_L(rho_L, rho_R, Ls.r, a), rRh = mausm_phi_R(rho_L, rho_R, Rs.r, a);
  double uLh = mausm_phi_L(u_LHS, u_RHS, Ls.u, a), uRh = mausm_phi_R(u_LHS, u_RHS, Rs.u, a);
  double vLh = mausm_phi_L(v_LHS, v_RHS, Ls.v, a), vRh = mausm_phi_R(v_LHS, v_RHS, Rs.v, a);
  double pLh = mausm_phi_L(p_L, p_R, Ls.p, a), pRh = mausm_phi_R(p_L, p_R, Rs.p, a);
  double H_Lh = (g / (g - 1.0)) * (pLh / rLh) + 0.5 * (uLh * uLh + vLh * vLh);
  double H_Rh = (g / (g - 1.0)) * (pRh / rRh) + 0.5 * (uRh * uRh + vRh * vRh);
  double mL = Mb_L * c_half * rLh;
  double mR = Mb_R * c_half * rRh;
  if (fabs(mL + mR) < EPSF) { mL = 0.0; mR = 0.0; }
  F[0] = mL + mR;
  double tx = (mL * uLh) + (mR * uRh), px = (P_L_plus * nx * p_L) + (P_R_minus * nx * p_R);
  F[1] = fabs(tx) < EPSF ? px : tx + px;
  double ty = (mL * vLh) + (mR * vRh), py = (P_L_plus * ny * p_L) + (P_R_minus * ny * p_R);
  F[2] = fabs(ty) < EPSF ? py : ty + py;
  F[3] = (mL * H_Lh) + (mR * H_Rh);
  if (fabs(F[3]) < EPSF) F[3] = 0.0;
}

/* SLAU family, slau_solver.fypp:332-490.  pc (SD variants) = delta_p1..6 cell pairs:
 * pc[0..5] = first cell of each pair, pc[6..11] = second cell. */
static void flux_slau(const cato_config* c, double nx, double ny, prim_t Lq, prim_t Rq,
                      const double pc[12], double F[4]) {
  const double g = c->gamma;
  const double THRESHOLD = 5e-3, C_SD1 = 0.01;
  const int variant = c->flux;
  double rho_L = Lq.r, u_L = Lq.u, v_L = Lq.v, p_L = Lq.p;
  double rho_R = Rq.r, u_R = Rq.u, v_R = Rq.v, p_R = Rq.p;
  double Vp = u_L * nx + v_L * ny;
  double Vm = u_R * nx + v_R * ny;
  double c_plus = sqrt(g * p_L / rho_L);
  double c_minus = sqrt(g * p_R / rho_R);
  double c_bar = 0.5 * (c_plus + c_minus);
  double V_n_bar = (rho_L * fabs(Vp) + rho_R * fabs(Vm)) / (rho_L + rho_R);
  double M_hat = dmin(1.0, sqrt(0.5 * (u_L * u_L + v_L * v_L + u_R * u_R + v_R * v_R)) / c_bar);
  double Chi = (1.0 - M_hat) * (1.0 - M_hat);
  double M_bar = V_n_bar / c_bar;
  double p_bar = 0.5 * (p_L + p_R);
  double rho_bar = 0.5 * (rho_L + rho_R);
  double M_plus = Vp / c_bar;
  double M_minus = Vm / c_bar;
  double B_plus, B_minus;
  if (fabs(M_plus) < 1.0) B_plus = 0.25 * (2.0 - M_plus) * ((M_plus + 1.0) * (M_plus + 1.0));
  else B_plus = 0.5 * (1.0 + fsign1(M_plus));
  if (fabs(M_minus) < 1.0) B_minus = 0.25 * (2.0 + M_minus) * ((M_minus - 1.0) * (M_minus - 1.0));
  else B_minus = 0.5 * (1.0 + fsign1(-M_minus));
  double delta_p = p_R - p_L;
  if (fabs(delta_p) < EPS || fabs(delta_p) < THRESHOLD * p_bar) delta_p = 0.0;
  double delta_rho = rho_R - rho_L;
  if (fabs(delta_rho) < EPS) delta_rho = 0.0;
  double delta_B = B_plus - B_minus;
  if (fabs(delta_B) < EPS) delta_B = 0.0;
  double pLmR = p_L - p_R;
  if (fabs(pLmR) < EPS) pLmR = 0.0;
  double theta = 0.0;
  if (variant == CATO_FLUX_SD_SLAU || variant == CATO_FLUX_SD_SLAU2) {
    double dpk[6];
    for (int k = 0; k < 6; ++k) {
      dpk[k] = fabs(pc[k] - pc[6 + k]);
      if (dpk[k] < EPS || dpk[k] < THRESHOLD * p_bar) dpk[k] = 0.0;
    }
    double m6 = dmax(dmax(dmax(dmax(dmax(dpk[0], dpk[1]), dpk[2]), dpk[3]), dpk[4]), dpk[5]);
    double dp_max = dmax(fabs(delta_p), m6);
    double ratio = ((C_SD1 * fabs(delta_p) / p_bar) + C_SD1) / ((dp_max / p_bar) + C_SD1);
    theta = dmin(1.0, ratio * ratio) * dmax(0.0, 1.0 - fabs(M_bar));
  }
  double p_tilde;
  if (variant == CATO_FLUX_SLAU || variant == CATO_FLUX_SD_SLAU)
    p_tilde = (p_bar + 0.5 * delta_B * pLmR) + (1.0 - Chi) * (B_plus + B_minus - 1.0) * p_bar;
  else
    p_tilde = p_bar + (0.5 * delta_B * pLmR) +
              sqrt(0.5 * (u_L * u_L + v_L * v_L + u_R * u_R + v_R * v_R)) *
                  (B_plus + B_minus - 1.0) * rho_bar * c_bar;
  double gg = -(dmax(dmin(M_plus, 0.0), -1.0) * dmin(dmax(M_minus, 0.0), 1.0));
  double mf;
  if (variant == CATO_FLUX_SLAU || variant == CATO_FLUX_SLAU2)
    mf = 0.5 * ((rho_L * Vp) + (rho_R * Vm) - fabs(V_n_bar) * delta_rho) * (1.0 - gg) -
         ((Chi / (2.0 * c_bar)) * delta_p);
  else
    mf = 0.5 * ((rho_L * Vp) + (rho_R * Vm) - fabs(V_n_bar) * delta_rho) * (1.0 - gg) -
         ((theta / (2.0 * c_bar)) * delta_p);
  double mL = 0.5 * (mf + fabs(mf));
  double mR = 0.5 * (mf - fabs(mf));
  double H_L = (g / (g - 1.0)) * (p_L / rho_L) + 0.5 * (u_L * u_L + v_L * v_L);
  double H_R = (g / (g - 1.0)) * (p_R / rho_R) + 0.5 * (u_R * u_R + v_R * v_R);
  F[0] = mL + mR;
  F[1] = (mL * u_L) + (mR * u_R) + p_tilde * nx;
  F[2] = (mL * v_L) + (mR * v_R) + p_tilde * ny;
  F[3] = (mL * H_L) + (mR * H_R);
}

/* f_h pressure sensor, roe_solver.fypp:519-527 */
static double roe_f_h(double pL, double pR) {
  double ratio = fabs(pR - pL) / (dmin(pR, pL) + 1e-16);
  return (ratio < 1.0) ? 0.0 : 1.0;
}
/* entropy_correction, roe_solver.fypp:529-536 (used only with the Harten flag; unpinned) */
static double roe_entropy_correction(double z, double dd) {
  if (z > dd) return z;
  return 0.5 * (z * z + dd * dd) / dd;
}

/* Roe, roe_solver.fypp:420-512.  pc = the five f_h pressure pairs (first cells pc[0..4],
 * second cells pc[5..9]). */
static void flux_roe(const cato_config* c, double nx, double ny, prim_t Lq, prim_t Rq,
                     const double pc[10], double F[4]) {
  const double g = c->gamma;
  double rl = fabs(Lq.r), ul = Lq.u, vl = Lq.v, pl = fabs(Lq.p);
  double hl = (g / (g - 1.0)) * (pl / rl) + 0.5 * (ul * ul + vl * vl);
  double rr = fabs(Rq.r), ur = Rq.u, vr = Rq.v, pr = fabs(Rq.p);
  double hr = (g / (g - 1.0)) * (pr / rr) + 0.5 * (ur * ur + vr * vr);
  double rav = sqrt(rl * rr);
  double gam1 = g - 1.0;
  double dd = rav / rl;
  double dd1 = 1.0 / (1.0 + dd);
  double uav = (ul + dd * ur) * dd1;
  double vav = (vl + dd * vr) * dd1;
  double hav = (hl + dd * hr) * dd1;
  double q2a = 0.5 * (uav * uav + vav * vav);
  double c2a = gam1 * (hav - q2a);
  double cav = sqrt(c2a);
  double uv = uav * nx + vav * ny;
  double du = (ur - ul) * nx + (vr - vl) * ny;
  double du_trans = -((ur - ul) * ny) + (vr - vl) * nx;
  double cs_R = sqrt(g * pr / rr);
  double cs_L = sqrt(g * pl / rl);
  double h1 = fabs(dmin(uv - cav, (ul * nx + vl * ny) - cs_L));
  double h2 = fabs(uv);
  double h4 = fabs(dmax(uv + cav, (ur * nx + vr * ny) + cs_R));
  double eabs1 = h1, eabs2 = h2, eabs4 = h4;
  if (c->roe_entropy_fix == CATO_ROE_HARTEN) {
    double delta = c->harten_delta * cav;
    eabs1 = roe_entropy_correction(h1, delta);
    eabs2 = roe_entropy_correction(h2, delta);
    eabs4 = roe_entropy_correction(h4, delta);
  }
  h1 = rav * cav * du;
  h2 = eabs1 * (pr - pl - h1) / (2.0 * c2a);
  double h3 = eabs2 * (rr - rl - (pr - pl) / c2a);
  h4 = eabs2 * rav;
  double h5 = eabs4 * (pr - pl + h1) / (2.0 * c2a);
  double psi = fabs(cs_R - cs_L) / dmax(cs_R, cs_L);
  double FR[4] = {rr * uv, rr * ur * uv + nx * pr, rr * vr * uv + ny * pr, rr * hr * uv};
  double FL[4] = {rl * uv, rl * ul * uv + nx * pl, rl * vl * uv + ny * pl, rl * hl * uv};
  double rmt[4];
  rmt[0] = (h2 + h3 + h5);
  rmt[1] = (h2 * (uav - cav * nx) + h3 * uav + h4 * (ur - ul - du * nx) + h5 * (uav + cav * nx));
  rmt[2] = (h2 * (vav - cav * ny) + h3 * vav + h4 * (vr - vl - du * ny) + h5 * (vav + cav * ny));
  rmt[3] = (h2 * (hav - cav * uv) + h3 * q2a + h4 * (uav * (ur - ul) + vav * (vr - vl) - uv * du) +
            h5 * (hav + cav * uv));
  for (int k = 0; k < 4; ++k) F[k] = 0.5 * (FR[k] + FL[k] - rmt[k]);
  double fmax = 0.0;
  for (int k = 0; k < 5; ++k) fmax = dmax(fmax, roe_f_h(pc[k], pc[5 + k]));
  /* maxval(f_p) over {0,1}: the 5 values are non-negative so starting at 0 is exact */
  F[1] = F[1] - 0.5 * fmax * rav * cav * (-(du_trans * ny) + psi * du * nx);
  F[2] = F[2] - 0.5 * fmax * rav * cav * (du_trans * nx + psi * du * ny);
}

/* AUSM+-up split polynomials, ausm_plus_solver.f90:394-485 */
static double m1p(double M) { return 0.5 * (M + fabs(M)); }
static double m1m(double M) { return 0.5 * (M - fabs(M)); }
static double m2p(double M) { return 0.25 * ((M + 1.0) * (M + 1.0)); }
static double m2m(double M) { return -(0.25 * ((M - 1.0) * (M - 1.0))); }
static double m4p(double M, double beta) {
  if (fabs(M) >= 1.0) return m1p(M);
  return m2p(M) * (1.0 - 16.0 * beta * m2m(M));
}
static double m4m(double M, double beta) {
  if (fabs(M) >= 1.0) return m1m(M);
  return m2m(M) * (1.0 + 16.0 * beta * m2p(M));
}
static double p5p(double M, double alpha) {
  if (fabs(M) >= 1.0) return m1p(M) / M;
  return m2p(M) * ((2.0 - M) - 16.0 * alpha * M * m2m(M));
}
static double p5m(double M, double alpha) {
  if (fabs(M) >= 1.0) return m1m(M) / M;
  return m2m(M) * ((-2.0 - M) + 16.0 * alpha * M * m2p(M));
}

/* AUSM+-up (basic): interface_state, ausm_plus_solver.f90:499-643, and the upwinding of the
 * commented driver :313-325.  Unpinned: the reference driver is commented out. */
static void flux_ausm_up(const cato_config* c, double nx, double ny, prim_t Lq, prim_t Rq,
                         double F[4]) {
  const double g = c->gamma;
  const double alpha = 3.0 / 16.0; /* pressure_split_alpha, :51 */
  double gamma_factor = ((2.0 * (g - 1.0)) / (g + 1.0));
  double vel_L = Lq.u * nx + Lq.v * ny;
  double vel_R = Rq.u * nx + Rq.v * ny;
  double H_L = (Lq.p / Lq.r) * (g / (g - 1.0)) + 0.5 * (Lq.u * Lq.u + Lq.v * Lq.v);
  double H_R = (Rq.p / Rq.r) * (g / (g - 1.0)) + 0.5 * (Rq.u * Rq.u + Rq.v * Rq.v);
  double a_crit_L = sqrt(gamma_factor * fabs(H_L));
  double a_crit_R = sqrt(gamma_factor * fabs(H_R));
  double a_circ_L = (a_crit_L * a_crit_L) / dmax(a_crit_L, vel_L);
  double a_circ_R = (a_crit_R * a_crit_R) / dmax(a_crit_R, -vel_R);
  double a_half = dmin(a_circ_L, a_circ_R);
  double M_L = vel_L / a_half;
  double M_R = vel_R / a_half;
  double M_bar_sq = 0.5 * (M_L + M_R); /* as written at :585 */
  double M_plus = m4p(M_L, c->ausm_beta);
  double M_minus = m4m(M_R, c->ausm_beta);
  double rho_half = 0.5 * (Rq.r + Lq.r);
  double M_p;
  if (fabs(Rq.p - Lq.p) < EPS) M_p = 0.0;
  else
    M_p = -(c->ausm_kp * dmax(1.0 - c->ausm_sigma * M_bar_sq, 0.0) *
            ((Rq.p - Lq.p) / (rho_half * (a_half * a_half))));
  double M_sum = M_plus + M_minus;
  if (fabs(M_sum) < 1e-13) M_sum = 0.0;
  double M_half = M_sum + M_p;
  if (fabs(M_half) < 1e-13) M_half = 0.0;
  double P_plus = p5p(M_L, alpha);
  double P_minus = p5m(M_R, alpha);
  double p_u;
  if (fabs(vel_R - vel_L) < EPS) p_u = 0.0;
  else p_u = -(c->ausm_ku * P_plus * P_minus * (Lq.r + Rq.r) * a_half * (vel_R - vel_L));
  double p_half = P_plus * Lq.p + P_minus * Rq.p + p_u;
  if (M_half > 0.0) {
    double mf = M_half * a_half * Lq.r;
    F[0] = mf;
    F[1] = mf * Lq.u + (nx * p_half);
    F[2] = mf * Lq.v + (ny * p_half);
    F[3] = mf * H_L;
  } else {
    double mf = M_half * a_half * Rq.r;
    F[0] = mf;
    F[1] = mf * Rq.u + (nx * p_half);
    F[2] = mf * Rq.v + (ny * p_half);
    F[3] = mf * H_R;
  }
}

/* HLLC (Toro, "Riemann Solvers and Numerical Methods for Fluid Dynamics", 3rd ed., 2009,
 * Sec. 10.4-10.6): PVRS pressure estimate and pressure-based wave speeds, as set up by the
 * unfinished reference stub hllc_solver.fypp:345-353.  Unpinned. */
static void flux_hllc(const cato_config* c, int dir, prim_t Lq, prim_t Rq, double F[4]) {
  const double g = c->gamma;
  double qnL = dir == 0 ? Lq.u : Lq.v, qtL = dir == 0 ? Lq.v : Lq.u;
  double qnR = dir == 0 ? Rq.u : Rq.v, qtR = dir == 0 ? Rq.v : Rq.u;
  double cL = sqrt(g * Lq.p / Lq.r), cR = sqrt(g * Rq.p / Rq.r);
  double rho_bar = 0.5 * (Lq.r + Rq.r), c_bar = 0.5 * (cL + cR);
  double p_pvrs = 0.5 * (Lq.p + Rq.p) - 0.5 * (qnR - qnL) * rho_bar * c_bar;
  double p_star = dmax(0.0, p_pvrs);
  double gf = (g + 1.0) / (2.0 * g);
  double qL = (p_star <= Lq.p) ? 1.0 : sqrt(1.0 + gf * (p_star / Lq.p - 1.0));
  double qR = (p_star <= Rq.p) ? 1.0 : sqrt(1.0 + gf * (p_star / Rq.p - 1.0));
  double SL = qnL - cL * qL, SR = qnR + cR * qR;
  double EL = Lq.p / (g - 1.0) + 0.5 * Lq.r * (Lq.u * Lq.u + Lq.v * Lq.v);
  double ER = Rq.p / (g - 1.0) + 0.5 * Rq.r * (Rq.u * Rq.u + Rq.v * Rq.v);
  double S_star = (Rq.p - Lq.p + Lq.r * qnL * (SL - qnL) - Rq.r * qnR * (SR - qnR)) /
                  (Lq.r * (SL - qnL) - Rq.r * (SR - qnR));
  /* flux components in (normal, tangential) frame: mass, normal mom, tangential mom, energy */
  double FLn[4] = {Lq.r * qnL, Lq.r * qnL * qnL + Lq.p, Lq.r * qnL * qtL, qnL * (EL + Lq.p)};
  double FRn[4] = {Rq.r * qnR, Rq.r * qnR * qnR + Rq.p, Rq.r * qnR * qtR, qnR * (ER + Rq.p)};
  double Fn[4];
  if (SL >= 0.0) {
    memcpy(Fn, FLn, sizeof Fn);
  } else if (S_star >= 0.0) {
    double f = Lq.r * (SL - qnL) / (SL - S_star);
    double Us[4] = {f, f * S_star, f * qtL,
                    f * (EL / Lq.r + (S_star - qnL) * (S_star + Lq.p / (Lq.r * (SL - qnL))))};
    double Uk[4] = {Lq.r, Lq.r * qnL, Lq.r * qtL, EL};
    for (int k = 0; k < 4; ++k) Fn[k] = FLn[k] + SL * (Us[k] - Uk[k]);
  } else if (SR > 0.0) {
    double f = Rq.r * (SR - qnR) / (SR - S_star);
    double Us[4] = {f, f * S_star, f * qtR,
                    f * (ER / Rq.r + (S_star - qnR) * (S_star + Rq.p / (Rq.r * (SR - qnR))))};
    double Uk[4] = {Rq.r, Rq.r * qnR, Rq.r * qtR, ER};
    for (int k = 0; k < 4; ++k) Fn[k] = FRn[k] + SR * (Us[k] - Uk[k]);
  } else {
    memcpy(Fn, FRn, sizeof Fn);
  }
  F[0] = Fn[0];
  F[1] = dir == 0 ? Fn[1] : Fn[2];
  F[2] = dir == 0 ? Fn[2] : Fn[1];
  F[3] = Fn[3];
}

/* One edge flux from the reconstructed states; the cell pressures p (BC-filled) feed the
 * shock sensors.  Edge (i,j) sits between cells (i,j) and (i+1,j) [dir 0] or (i,j+1) [dir 1]. */
#define PN(n, t) (dir == 0 ? AT(p, i + (n), j + (t)) : AT(p, i + (t), j + (n)))
static void edge_flux(dims_t d, const cato_config* c, int dir, const double* p, int i, int j,
                      prim_t Lq, prim_t Rq, prim_t Ls, prim_t Rs, double F[4]) {
  /* Cartesian edge normals: exactly (1,0) for i-edges and (0,1) for j-edges
   * (quad_cell.f90:193-229 evaluated on axis-aligned cells) */
  double nx = dir == 0 ? 1.0 : 0.0, ny = dir == 0 ? 0.0 : 1.0;
  switch (c->flux) {
    case CATO_FLUX_AUSMPW_PLUS:
    case CATO_FLUX_M_AUSMPW_PLUS: {
      /* get_f arguments, ausmpw_plus_solver.fypp:430-442 (the same cells in
       * m_ausmpw_plus_solver.fypp:669-679) */
      double pc[4];
      if (dir == 0) {
        pc[0] = AT(p, i, j - 1); pc[1] = AT(p, i + 1, j - 1);
        pc[2] = AT(p, i, j + 1); pc[3] = AT(p, i + 1, j + 1);
      } else {
        pc[0] = AT(p, i + 1, j); pc[1] = AT(p, i + 1, j + 1);
        pc[2] = AT(p, i - 1, j); pc[3] = AT(p, i - 1, j + 1);
      }
      if (c->flux == CATO_FLUX_M_AUSMPW_PLUS) flux_mausmpw(c, dir, nx, ny, Lq, Rq, Ls, Rs, pc, F);
      else flux_ausmpw(c, dir, nx, ny, Lq, Rq, pc, F);
      break;
    }
    case CATO_FLUX_SLAU:
    case CATO_FLUX_SLAU2:
    case CATO_FLUX_SD_SLAU:
    case CATO_FLUX_SD_SLAU2: {
      /* delta_p1..6 cell pairs, slau_solver.fypp:410-430 */
      double pc[12] = {0};
      if (c->flux == CATO_FLUX_SD_SLAU || c->flux == CATO_FLUX_SD_SLAU2) {
        if (dir == 0) {
          pc[0] = AT(p, i, j + 1);     pc[6] = AT(p, i, j);
          pc[1] = AT(p, i - 1, j);     pc[7] = AT(p, i, j);
          pc[2] = AT(p, i, j - 1);     pc[8] = AT(p, i, j);
          pc[3] = AT(p, i + 1, j - 1); pc[9] = AT(p, i + 1, j);
          pc[4] = AT(p, i + 2, j);     pc[10] = AT(p, i + 1, j);
          pc[5] = AT(p, i + 1, j + 1); pc[11] = AT(p, i + 1, j);
        } else {
          pc[0] = AT(p, i - 1, j);     pc[6] = AT(p, i, j);
          pc[1] = AT(p, i, j - 1);     pc[7] = AT(p, i, j);
          pc[2] = AT(p, i + 1, j);     pc[8] = AT(p, i, j);
          pc[3] = AT(p, i + 1, j + 1); pc[9] = AT(p, i, j + 1);
          pc[4] = AT(p, i, j + 2);     pc[10] = AT(p, i, j + 1);
          pc[5] = AT(p, i - 1, j + 1); pc[11] = AT(p, i, j + 1);
        }
      }
      flux_slau(c, nx, ny, Lq, Rq, pc, F);
      break;
    }
    case CATO_FLUX_ROE: {
      /* f_p pairs, roe_solver.fypp:495-508 */
      double pc[10];
      if (dir == 0) {
        pc[0] = AT(p, i, j);     pc[5] = AT(p, i + 1, j);
        pc[1] = AT(p, i, j);     pc[6] = AT(p, i, j + 1);
        pc[2] = AT(p, i, j);     pc[7] = AT(p, i, j - 1);
        pc[3] = AT(p, i, j + 1); pc[8] = AT(p, i + 1, j + 1);
        pc[4] = AT(p, i, j - 1); pc[9] = AT(p, i + 1, j - 1);
      } else {
        pc[0] = AT(p, i, j);     pc[5] = AT(p, i, j + 1);
        pc[1] = AT(p, i, j);     pc[6] = AT(p, i - 1, j);
        pc[2] = AT(p, i, j);     pc[7] = AT(p, i + 1, j);
        pc[3] = AT(p, i, j + 1); pc[8] = AT(p, i - 1, j + 1);
        pc[4] = AT(p, i, j + 1); pc[9] = AT(p, i + 1, j + 1);
      }
      flux_roe(c, nx, ny, Lq, Rq, pc, F);
      break;
    }
    case CATO_FLUX_AUSM_PLUS_UP: flux_ausm_up(c, nx, ny, Lq, Rq, F); break;
    case CATO_FLUX_HLLC: flux_hllc(c, dir, Lq, Rq, F); break;
    default: F[0] = F[1] = F[2] = F[3] = NAN;
  }
}
#undef PN

/* flux_split_edges, flux_solver.f90:252-425 for one cell and one conserved variable k. */
static double divergence(double Fi, double Fim, double Fj, double Fjm, const geom_t* g) {
  const double REL_TOL = 1e-14;
  const double near0 = 5.0 * TINY; /* near_zero, flux_solver.f90:461-474 */
  double mi = dmax(dmax(fabs(Fi), fabs(Fim)), 1.0);
  double mj = dmax(dmax(fabs(Fj), fabs(Fjm)), 1.0);
  double a = ((Fi / mi * g->l[1]) + (-(Fim / mi * g->l[3]))) * mi;
  double b = ((Fj / mj * g->l[2]) + (-(Fjm / mj * g->l[0]))) * mj;
  if (fabs(a) < mi * REL_TOL) a = 0.0;
  if (fabs(b) < mj * REL_TOL) b = 0.0;
  double s = a + b;
  if (fabs(s) < near0) s = 0.0;
  return (-s) / g->vol;
}

/* flux_solver_t%solve for the edge-split solvers (e.g. slau_solver.fypp:123-249): BCs on the
 * primitives, reconstruction, edge fluxes, flux divergence.  d_* are halo-padded, ghosts 0.
 * `cells` holds per-cell metrics (rect_cells) or is NULL for the uniform dx x dy grid. */
static int solve_geo(const cato_config* c, const geom_t* cells, const pbc_ctx_t* pc, double* rho,
                     double* u, double* v, double* p, double* drho, double* drhou, double* drhov,
                     double* drhoE) {
  dims_t d = mkdims(c);
  geom_t geo = uniform_geom(c);
  apply_bc_at(c, pc, rho, u, v, p);
  double* iflux = (double*)malloc(sizeof(double) * 4 * (size_t)(d.ni + 1) * d.nj);
  double* jflux = (double*)malloc(sizeof(double) * 4 * (size_t)d.ni * (d.nj + 1));
  if (!iflux || !jflux) { free(iflux); free(jflux); return CATO_ERR_OOM; }
  const double* q[4] = {rho, u, v, p};
  /* i-direction edges (0:ni, 1:nj) */
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= d.nj; ++j)
    for (int i = 0; i <= d.ni; ++i) {
      double L[4], R[4], Ls[4] = {0}, Rs[4] = {0};
      for (int k = 0; k < 4; ++k) edge_recon(d, c->limiter, q[k], 0, i, j, &L[k], &R[k]);
      if (c->flux == CATO_FLUX_M_AUSMPW_PLUS) /* the superbee edge states, :163-167 */
        for (int k = 0; k < 4; ++k) edge_recon(d, CATO_LIM_SUPERBEE, q[k], 0, i, j, &Ls[k], &Rs[k]);
      prim_t Lq = {L[0], L[1], L[2], L[3]}, Rq = {R[0], R[1], R[2], R[3]};
      prim_t Lsq = {Ls[0], Ls[1], Ls[2], Ls[3]}, Rsq = {Rs[0], Rs[1], Rs[2], Rs[3]};
      edge_flux(d, c, 0, p, i, j, Lq, Rq, Lsq, Rsq, &IF(iflux, 0, i, j));
    }
  /* j-direction edges (1:ni, 0:nj) */
#pragma omp parallel for schedule(static)
  for (int j = 0; j <= d.nj; ++j)
    for (int i = 1; i <= d.ni; ++i) {
      double L[4], R[4], Ls[4] = {0}, Rs[4] = {0};
      for (int k = 0; k < 4; ++k) edge_recon(d, c->limiter, q[k], 1, i, j, &L[k], &R[k]);
      if (c->flux == CATO_FLUX_M_AUSMPW_PLUS)
        for (int k = 0; k < 4; ++k) edge_recon(d, CATO_LIM_SUPERBEE, q[k], 1, i, j, &Ls[k], &Rs[k]);
      prim_t Lq = {L[0], L[1], L[2], L[3]}, Rq = {R[0], R[1], R[2], R[3]};
      prim_t Lsq = {Ls[0], Ls[1], Ls[2], Ls[3]}, Rsq = {Rs[0], Rs[1], Rs[2], Rs[3]};
      edge_flux(d, c, 1, p, i, j, Lq, Rq, Lsq, Rsq, &JF(jflux, 0, i, j));
    }
  double* out[4] = {drho, drhou, drhov, drhoE};
  size_t n = nfield(d);
  for (int k = 0; k < 4; ++k) memset(out[k], 0, n * sizeof(double));
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= d.nj; ++j)
    for (int i = 1; i <= d.ni; ++i)
      for (int k = 0; k < 4; ++k)
        AT(out[k], i, j) = divergence(IF(iflux, k, i, j), IF(iflux, k, i - 1, j),
                                      JF(jflux, k, i, j), JF(jflux, k, i, j - 1),
                                      cells ? &cells[(size_t)(j - 1) * d.ni + (i - 1)] : &geo);
  free(iflux);
  free(jflux);
  return 0;
}

int oracle_solve(const cato_config* c, double* rho, double* u, double* v, double* p,
                 double* drho, double* drhou, double* drhov, double* drhoE) {
  return solve_geo(c, NULL, NULL, rho, u, v, p, drho, drhou, drhov, drhoE);
}

int oracle_solve_pbc(const cato_config* c, int32_t n, const double* t, const double* pt,
                     const double* rhot, double time, double* rho, double* u, double* v, double* p,
                     double* drho, double* drhou, double* drhov, double* drhoE) {
  if (oracle_config_check(c) != CATO_OK) return CATO_ERR_CONFIG;
  pbc_ctx_t pc = {n, t, pt, rhot, time};
  return solve_geo(c, NULL, &pc, rho, u, v, p, drho, drhou, drhov, drhoE);
}

int oracle_solve_rect(const cato_config* c, const double* x_nodes, const double* y_nodes,
                      double* rho, double* u, double* v, double* p, double* drho, double* drhou,
                      double* drhov, double* drhoE) {
  if (oracle_config_check(c) != CATO_OK) return CATO_ERR_CONFIG;
  geom_t* cells = rect_cells(c->ni, c->nj, x_nodes, y_nodes);
  if (!cells) return CATO_ERR_ARG;
  int rc = solve_geo(c, cells, NULL, rho, u, v, p, drho, drhou, drhov, drhoE);
  free(cells);
  return rc;
}

/* ------------------------------------------------------------------------------------------ */
/* fluid_t                                                                                     */
/* ------------------------------------------------------------------------------------------ */
struct oracle_fluid {
  cato_config c;
  dims_t d;
  geom_t geo;
  geom_t* cells; /* per-cell metrics of a rectilinear grid (rect_cells), NULL if uniform */
  /* pressure-input table (NULL: the configuration's constants) and the flux-solver clock of the
   * persistent fluid (flux solvers add dt to their time before applying the BCs, e.g.
   * slau_solver.fypp:168; copies of a fluid re-initialise theirs to the fluid's time,
   * assign_fluid mod_fluid.f90:706) */
  double* pbc_tab;
  int pbc_n;
  /* energy source term (mod_source.f90): configuration, table (time, value, critical
   * density), the grid nodes for the centroids, and q_dot_h of the current step */
  int src_on;
  cato_energy_source src;
  double* src_tab;
  int src_n;
  double* xn;
  double* yn;
  double* srcq;
  double solver_time;
  double bc_time;    /* boundary time of the residual being evaluated */
  /* conserved (U) and derived (u, v, p, cs) of the current state */
  double *rho, *rhou, *rhov, *rhoE, *u, *v, *p, *cs;
  /* scratch: stage states, primitive copies for the solver, residuals */
  double* st[3][4];  /* stage conserved U_1, U_2 / U_prev, U_curr */
  double* sp[4];     /* primitives handed to the solver (BCs write their ghosts) */
  double* L[4];
  double time, dt;
  int64_t iteration;
  double conv[4];   /* calculate_convergence of the last step */
  int conv_valid;
  /* allow_subcycle / subcycle_tolerance (mod_fluid.f90:98-99, 856-887) */
  int subcycle;
  double subcycle_tol;
  /* a slab of a row-split grid: fills the ghost rows beyond its exchange sides with the
   * neighbouring slabs' rows of the same stage before the boundary conditions (time_derivative
   * calls sync_fields on rho, u, v, p: mod_fluid.f90:452-458, 485; field_2d.f90:551-654) */
  oracle_exchange_fn xchg;
  void* xchg_user;
};

static void source_field(oracle_fluid* f);

static double* falloc(dims_t d) { return (double*)calloc(nfield(d), sizeof(double)); }

oracle_fluid* oracle_create(const cato_config* c) {
  if (oracle_config_check(c) != CATO_OK) return NULL;
  oracle_fluid* f = (oracle_fluid*)calloc(1, sizeof(*f));
  f->c = *c;
  f->d = mkdims(c);
  f->geo = uniform_geom(c);
  double** all[] = {&f->rho, &f->rhou, &f->rhov, &f->rhoE, &f->u, &f->v, &f->p, &f->cs};
  for (size_t k = 0; k < sizeof all / sizeof all[0]; ++k) *all[k] = falloc(f->d);
  for (int s = 0; s < 3; ++s)
    for (int k = 0; k < 4; ++k) f->st[s][k] = falloc(f->d);
  for (int k = 0; k < 4; ++k) { f->sp[k] = falloc(f->d); f->L[k] = falloc(f->d); }
  return f;
}

void oracle_destroy(oracle_fluid* f) {
  if (!f) return;
  double* all[] = {f->rho, f->rhou, f->rhov, f->rhoE, f->u, f->v, f->p, f->cs};
  for (size_t k = 0; k < sizeof all / sizeof all[0]; ++k) free(all[k]);
  for (int s = 0; s < 3; ++s)
    for (int k = 0; k < 4; ++k) free(f->st[s][k]);
  for (int k = 0; k < 4; ++k) { free(f->sp[k]); free(f->L[k]); }
  free(f->cells);
  free(f->pbc_tab);
  free(f->src_tab);
  free(f->xn);
  free(f->yn);
  free(f->srcq);
  free(f);
}

/* conserved -> primitive + sound speed + Mach filter, per interior cell:
 * eos%conserved_to_primitive (equation_of_state.f90:297-314) through the field operators
 * (field_2d_cpu_operators.f90:84-420: +/- flush |x|<eps, field/field returns 0 if |lhs|<tiny),
 * eos%sound_speed (:269-278), and calculate_derived_quantities (mod_fluid.f90:564-591). */
static void derive_cell(double g, double r, double ru, double rv, double rE, double* u_out,
                        double* v_out, double* p_out, double* cs_out) {
  double g1 = g - 1.0;
  double u = (fabs(ru) < TINY) ? 0.0 : ru / r;
  double v = (fabs(rv) < TINY) ? 0.0 : rv / r;
  double e = (fabs(rE) < TINY) ? 0.0 : rE / r;
  double s = u * u + v * v;
  if (fabs(s) < EPS) s = 0.0;
  double h = s * 0.5;
  double dd = e - h;
  if (fabs(dd) < EPS) dd = 0.0;
  double p = (r * g1) * dd;
  double pr = (fabs(p) < TINY) ? 0.0 : p / r;
  double cs = sqrt(pr * g);
  double mu = (fabs(u) < TINY) ? 0.0 : u / cs;
  double mv = (fabs(v) < TINY) ? 0.0 : v / cs;
  if (fabs(mv) < 1e-13) v = 0.0;
  if (fabs(mu) < 1e-13) u = 0.0;
  *u_out = u;
  *v_out = v;
  *p_out = p;
  *cs_out = cs;
}

static void derive_all(oracle_fluid* f, double* const U[4], double* u, double* v, double* p,
                       double* cs) {
  dims_t d = f->d;
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= d.nj; ++j)
    for (int i = 1; i <= d.ni; ++i)
      derive_cell(f->c.gamma, AT(U[0], i, j), AT(U[1], i, j), AT(U[2], i, j), AT(U[3], i, j),
                  &AT(u, i, j), &AT(v, i, j), &AT(p, i, j), &AT(cs, i, j));
}

/* initialize_from_hdf5 + primitive_to_conserved (equation_of_state.f90:316-324 via the field
 * operators) + the initial sound speed (mod_fluid.f90:249; no Mach filter at start). */
int oracle_set_primitive(oracle_fluid* f, const double* rho, const double* u, const double* v,
                         const double* p) {
  dims_t d = f->d;
  double g1 = f->c.gamma - 1.0;
  double one_over_g1 = 1.0 / g1; /* field / real = field * (1/real), field_2d.f90:750-771 */
  for (int j = 1; j <= d.nj; ++j)
    for (int i = 1; i <= d.ni; ++i) {
      double r = AT(rho, i, j), uu = AT(u, i, j), vv = AT(v, i, j), pp = AT(p, i, j);
      AT(f->rho, i, j) = r;
      AT(f->u, i, j) = uu;
      AT(f->v, i, j) = vv;
      AT(f->p, i, j) = pp;
      AT(f->rhou, i, j) = uu * r;
      AT(f->rhov, i, j) = vv * r;
      double s = uu * uu + vv * vv;
      if (fabs(s) < EPS) s = 0.0;
      double E = pp * one_over_g1 + (r * 0.5) * s;
      if (fabs(E) < EPS) E = 0.0;
      AT(f->rhoE, i, j) = E;
      double pr = (fabs(pp) < TINY) ? 0.0 : pp / r;
      AT(f->cs, i, j) = sqrt(f->c.gamma * pr);
    }
  f->time = 0.0;
  f->solver_time = 0.0;
  f->iteration = 0;
  f->conv_valid = 0;
  /* initialize_from_hdf5's checks of the loaded state (mod_fluid.f90:352-360): pressure below
   * tiny, then density below tiny (comparisons with a NaN are false, as minval skips NaNs) */
  for (int j = 1; j <= d.nj; ++j)
    for (int i = 1; i <= d.ni; ++i)
      if (AT(p, i, j) < TINY) return CATO_NEG_PRESSURE;
  for (int j = 1; j <= d.nj; ++j)
    for (int i = 1; i <= d.ni; ++i)
      if (AT(rho, i, j) < TINY) return CATO_NEG_DENSITY;
  return 0;
}

/* fluid_t%set_time; as a fluid created at `time` (new_fluid(..., time)), its solver clock too */
int oracle_set_time(oracle_fluid* f, double time, int64_t iteration) {
  f->time = time;
  f->solver_time = time;
  f->iteration = iteration;
  return 0;
}

/* pressure-input target table (n = 0: the configuration's constants) */
int oracle_set_bc_table(oracle_fluid* f, int32_t n, const double* t, const double* p,
                        const double* rho) {
  free(f->pbc_tab);
  f->pbc_tab = NULL;
  f->pbc_n = 0;
  if (n <= 0) return 0;
  if (n < 2) return CATO_ERR_ARG;
  for (int k = 1; k < n; ++k)
    if (!(t[k] > t[k - 1])) return CATO_ERR_ARG;
  f->pbc_tab = (double*)malloc(sizeof(double) * 3 * (size_t)n);
  memcpy(f->pbc_tab, t, sizeof(double) * n);
  memcpy(f->pbc_tab + n, p, sizeof(double) * n);
  memcpy(f->pbc_tab + 2 * n, rho, sizeof(double) * n);
  f->pbc_n = n;
  return 0;
}

int oracle_set_conserved(oracle_fluid* f, const double* rho, const double* rho_u,
                         const double* rho_v, const double* rho_E) {
  dims_t d = f->d;
  for (int j = 1; j <= d.nj; ++j)
    for (int i = 1; i <= d.ni; ++i) {
      AT(f->rho, i, j) = AT(rho, i, j);
      AT(f->rhou, i, j) = AT(rho_u, i, j);
      AT(f->rhov, i, j) = AT(rho_v, i, j);
      AT(f->rhoE, i, j) = AT(rho_E, i, j);
    }
  double* U[4] = {f->rho, f->rhou, f->rhov, f->rhoE};
  derive_all(f, U, f->u, f->v, f->p, f->cs);
  f->conv_valid = 0;
  return 0;
}

/* get_timestep, mod_fluid.f90:518-562 (dx, dy = quad min_dx/min_dy, quad_cell.f90:119-123) */
double oracle_get_timestep(oracle_fluid* f) {
  dims_t d = f->d;
  double m = INFINITY;
  const double cfl = f->c.cfl;
  const geom_t* cells = f->cells;
  const geom_t geo = f->geo;
#pragma omp parallel for reduction(min : m) schedule(static)
  for (int j = 1; j <= d.nj; ++j)
    for (int i = 1; i <= d.ni; ++i) {
      const geom_t* g = cells ? &cells[(size_t)(j - 1) * d.ni + (i - 1)] : &geo;
      const double dx = g->dx, dy = g->dy;
      double cs = AT(f->cs, i, j);
      double t = cfl / (((fabs(AT(f->u, i, j)) + cs) / dx) + ((fabs(AT(f->v, i, j)) + cs) / dy));
      if (t < m) m = t;
    }
  return m;
}

/* L(U) for a state whose primitives are (pr, pu, pv, pp): time_derivative, mod_fluid.f90:460-516 */
static int residual(oracle_fluid* f, const double* pr, const double* pu, const double* pv,
                    const double* pp) {
  size_t n = nfield(f->d) * sizeof(double);
  memcpy(f->sp[0], pr, n);
  memcpy(f->sp[1], pu, n);
  memcpy(f->sp[2], pv, n);
  memcpy(f->sp[3], pp, n);
  if (f->xchg) f->xchg(f->xchg_user, f->sp[0], f->sp[1], f->sp[2], f->sp[3]);
  pbc_ctx_t pc = {f->pbc_n, f->pbc_tab, f->pbc_tab ? f->pbc_tab + f->pbc_n : NULL,
                  f->pbc_tab ? f->pbc_tab + 2 * f->pbc_n : NULL, f->bc_time};
  int rc = solve_geo(&f->c, f->cells, &pc, f->sp[0], f->sp[1], f->sp[2], f->sp[3], f->L[0],
                     f->L[1], f->L[2], f->L[3]);
  /* time_derivative (mod_fluid.f90:503): the source joins the energy equation */
  const dims_t d = f->d;
  if (f->src_on)
    for (int j = 1; j <= f->d.nj; ++j)
      for (int i = 1; i <= f->d.ni; ++i)
        AT(f->L[3], i, j) = AT(f->L[3], i, j) + f->srcq[(size_t)(j - 1) * f->d.ni + (i - 1)];
  return rc;
}

/* out = A + L*c with the field '+' flush (fluid operators mod_fluid.f90:609-669) */
static void stage_a(oracle_fluid* f, double* const out[4], double* const A[4], double cc) {
  dims_t d = f->d;
  for (int k = 0; k < 4; ++k)
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= d.nj; ++j)
      for (int i = 1; i <= d.ni; ++i) {
        double r = AT(A[k], i, j) + AT(f->L[k], i, j) * cc;
        if (fabs(r) < EPS) r = 0.0;
        AT(out[k], i, j) = r;
      }
}

/* out = (A*a + B*b) + L*c, each '+' flushed */
static void stage_b(oracle_fluid* f, double* const out[4], double* const A[4], double a,
                    double* const B[4], double b, double cc) {
  dims_t d = f->d;
  for (int k = 0; k < 4; ++k)
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= d.nj; ++j)
      for (int i = 1; i <= d.ni; ++i) {
        double s = AT(A[k], i, j) * a + AT(B[k], i, j) * b;
        if (fabs(s) < EPS) s = 0.0;
        double r = s + AT(f->L[k], i, j) * cc;
        if (fabs(r) < EPS) r = 0.0;
        AT(out[k], i, j) = r;
      }
}

/* calculate_convergence (mod_fluid.f90:1162-1205): L2 norm of the change from the first to the
 * last stage over the interior, relative to the first stage's norm (for rho u and rho v relative to
 * max(norm, 1)).  norm2 is restated as the square root of the plain sum of squares, summed in
 * (i fastest, then j) order; the Fortran intrinsic may scale its sum, which changes only the
 * last bits. */
static void convergence(oracle_fluid* f, double* const first[4], double* const last[4]) {
  dims_t d = f->d;
  for (int k = 0; k < 4; ++k) {
    double sd = 0.0, s0 = 0.0;
    for (int j = 1; j <= d.nj; ++j)
      for (int i = 1; i <= d.ni; ++i) {
        double a = AT(first[k], i, j), df = AT(last[k], i, j) - a;
        sd += df * df;
        s0 += a * a;
      }
    double n0 = sqrt(s0);
    if (k == 1 || k == 2) n0 = n0 > 1.0 ? n0 : 1.0;
    f->conv[k] = sqrt(sd) / n0;
  }
  f->conv_valid = 1;
}

int oracle_convergence(oracle_fluid* f, double out[4]) {
  if (!f->conv_valid) return CATO_ERR_STATE;
  for (int k = 0; k < 4; ++k) out[k] = f->conv[k];
  return CATO_OK;
}

/* Interior totals of the conserved variables (sum of U * cell volume): mass, x and y momentum
 * and energy in the domain, summed in (i fastest, then j) order. */
int oracle_conservation_sums(oracle_fluid* f, double out[4]) {
  dims_t d = f->d;
  double* U[4] = {f->rho, f->rhou, f->rhov, f->rhoE};
  for (int k = 0; k < 4; ++k) {
    double s = 0.0;
    for (int j = 1; j <= d.nj; ++j)
      for (int i = 1; i <= d.ni; ++i)
        s += f->cells ? AT(U[k], i, j) * f->cells[(size_t)(j - 1) * d.ni + (i - 1)].vol
                      : AT(U[k], i, j);
    out[k] = f->cells ? s : s * f->geo.vol;
  }
  return CATO_OK;
}

/* Rectilinear grid of node coordinates x(1..ni+1), y(1..nj+1); both NULL = uniform again. */
int oracle_set_rectilinear(oracle_fluid* f, const double* x_nodes, const double* y_nodes) {
  if (!x_nodes != !y_nodes) return CATO_ERR_ARG;
  geom_t* cells = NULL;
  if (x_nodes) {
    cells = rect_cells(f->d.ni, f->d.nj, x_nodes, y_nodes);
    if (!cells) return CATO_ERR_ARG;
  }
  free(f->cells);
  f->cells = cells;
  free(f->xn);
  free(f->yn);
  f->xn = f->yn = NULL;
  if (x_nodes) {
    f->xn = (double*)malloc(sizeof(double) * (f->d.ni + 1));
    f->yn = (double*)malloc(sizeof(double) * (f->d.nj + 1));
    memcpy(f->xn, x_nodes, sizeof(double) * (f->d.ni + 1));
    memcpy(f->yn, y_nodes, sizeof(double) * (f->d.nj + 1));
  }
  return CATO_OK;
}

/* energy source term: src NULL turns it off; n = 0 constant value, else the scaled table */
int oracle_set_energy_source(oracle_fluid* f, const cato_energy_source* src, int32_t n,
                             const double* t, const double* v, const double* crit) {
  free(f->src_tab);
  f->src_tab = NULL;
  f->src_on = 0;
  if (!src) return 0;
  if (n == 1 || n < 0) return CATO_ERR_ARG;
  for (int k = 1; k < n; ++k)
    if (!(t[k] > t[k - 1])) return CATO_ERR_ARG;
  if (n > 0) {
    f->src_tab = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    memcpy(f->src_tab, t, sizeof(double) * n);
    memcpy(f->src_tab + n, v, sizeof(double) * n);
    memcpy(f->src_tab + 2 * n, crit, sizeof(double) * n);
  }
  if (!f->srcq) f->srcq = (double*)calloc((size_t)f->d.ni * f->d.nj, sizeof(double));
  f->src = *src;
  f->src_n = n;
  f->src_on = 1;
  return 0;
}

/* The source field of a step starting now (f->time, f->rho): ni x nj values, i fastest. */
int oracle_source_field(oracle_fluid* f, double* out) {
  if (!f->src_on) return CATO_ERR_STATE;
  source_field(f);
  memcpy(out, f->srcq, sizeof(double) * (size_t)f->d.ni * f->d.nj);
  return 0;
}

/* quad_cell_t centroid (quad_cell.f90:145) of column i / row j (1-based) */
static double cen_x(const oracle_fluid* f, int i) {
  double x1 = f->xn ? f->xn[i - 1] : (double)(i - 1) * f->c.dx;
  double x2 = f->xn ? f->xn[i] : (double)i * f->c.dx;
  return (x2 + x1) / 2.0;
}
static double cen_y(const oracle_fluid* f, int j) {
  double y2 = f->yn ? f->yn[j - 1] : (double)(j - 1) * f->c.dy;
  double y3 = f->yn ? f->yn[j] : (double)j * f->c.dy;
  return (y3 + y2) / 2.0;
}

/* source_t%integrate (mod_source.f90:296-312) at the step start: find_deposition_location
 * (:314-353) and get_source_field (:355-425) into f->srcq */
static void source_field(oracle_fluid* f) {
  const dims_t d = f->d;
  const cato_energy_source* s = &f->src;
  const int n = f->src_n;
  const double t = f->time;
  /* the critical-density interpolator is only initialised from a table; uninitialised it
   * returns zero */
  double crit = n > 0 ? interp_1d(n, f->src_tab, f->src_tab + 2 * n, t) : 0.0;
  double x_center = 0.0;
  for (int i = d.ni; i >= 1; --i) {
    int any = 0;
    for (int j = 1; j <= d.nj; ++j) any |= AT(f->rho, i, j) > crit;
    if (any) {
      x_center = cen_x(f, i);
      break;
    }
  }
  double p_input;
  if (n == 0) {
    p_input = s->constant_value;
  } else {
    double tmax = f->src_tab[0];
    for (int k = 1; k < n; ++k) tmax = dmax(tmax, f->src_tab[k]);
    p_input = t <= tmax ? interp_1d(n, f->src_tab, f->src_tab + n, t) : 0.0;
  }
  p_input = p_input * s->multiplier;
  const double x0 = x_center;
  for (int j = 1; j <= d.nj; ++j)
    for (int i = 1; i <= d.ni; ++i) {
      double q = 0.0;
      if (fabs(p_input) > 0.0) {
        double x = cen_x(f, i), y = cen_y(f, j);
        switch (s->geometry) {
          case CATO_SRC_UNIFORM: q = p_input; break;
          case CATO_SRC_CONSTANT_XY:
            if (x < s->xhi && x > s->xlo && y < s->yhi && x > s->ylo) q = p_input;
            break;
          case CATO_SRC_GAUSSIAN_1D:
            if (fabs(x - x0) < s->fwhm_x * 5) {
              double a = ((x - x0) * (x - x0)) / (2 * (s->fwhm_x * s->fwhm_x));
              q = p_input * bc_exp(-powi(a, s->gaussian_order));
            }
            break;
          default: /* decay */
            if (x < x0) q = p_input * bc_exp(-bc_pow(x / x0, 1.5)) / bc_exp(-1.0);
            else q = p_input * bc_exp(-1e4 * (((x - x0) / x0) * ((x - x0) / x0)));
        }
      }
      f->srcq[(size_t)(j - 1) * d.ni + (i - 1)] = q;
    }
}

/* stage primitives (u, v, p, cs reused from the scratch solver arrays' neighbours) */
typedef struct {
  double *u, *v, *p, *cs;
} prims_t;

/* subcycle_check (mod_fluid.f90:856-887): with allow_subcycle, any L2 convergence norm of the
 * step above the tolerance repeats it with dt / 10 (a NaN norm does not) */
static int subcycle_check(const oracle_fluid* f) {
  if (!f->subcycle) return 0;
  for (int k = 0; k < 4; ++k)
    if (f->conv[k] > f->subcycle_tol) return 1;
  return 0;
}

double oracle_dt(const oracle_fluid* f) { return f->dt; }

int oracle_set_exchange(oracle_fluid* f, oracle_exchange_fn fn, void* user) {
  if (!f) return CATO_ERR_ARG;
  f->xchg = fn;
  f->xchg_user = user;
  return 0;
}

int oracle_set_subcycle(oracle_fluid* f, int allow, double tolerance) {
  f->subcycle = allow ? 1 : 0;
  f->subcycle_tol = tolerance;
  return 0;
}

/* fluid_t%integrate (mod_fluid.f90:411-450) for ssp_rk2 (:1081-1160), ssp_rk3 (:739-854) and
 * rk(m,n) (:889-1007); sanity check of the new state (:726-737) returns the reference codes. */
int oracle_integrate(oracle_fluid* f, double dt, int32_t* error_code) {
  dims_t d = f->d;
  f->dt = dt;
  f->iteration += 1;
  double* U[4] = {f->rho, f->rhou, f->rhov, f->rhoE};
  double *su[4], *sv[4], *spp[4], *scs[4];
  /* per-stage derived quantities (u, v, p, cs), allocated on demand */
  for (int s = 0; s < 4; ++s) { su[s] = falloc(d); sv[s] = falloc(d); spp[s] = falloc(d); scs[s] = falloc(d); }
  int rc = 0;
  /* boundary times: U%t advances the persistent fluid's solver clock; the stage copies U_1, U_2
   * (assigned from expressions led by U) restart theirs at U%time before adding dt */
  const double t_copy = f->time + dt;
  if (f->src_on) source_field(f); /* once per step, before the stages */
  if (f->c.rk == CATO_RK_SSP2) {
    double* U1[4] = {f->st[0][0], f->st[0][1], f->st[0][2], f->st[0][3]};
    double* U2[4] = {f->st[1][0], f->st[1][1], f->st[1][2], f->st[1][3]};
    /* the stages repeat with dt / 10 while subcycle_check asks for it (ssp_rk_2_2's loop,
     * mod_fluid.f90:1108-1140); U itself changes only after the loop */
    for (;;) {
      f->solver_time = f->solver_time + dt;
      f->bc_time = f->solver_time;
      rc |= residual(f, f->rho, f->u, f->v, f->p);
      stage_a(f, U1, U, dt);
      derive_all(f, U1, su[0], sv[0], spp[0], scs[0]);
      f->bc_time = f->time + dt;
      rc |= residual(f, U1[0], su[0], sv[0], spp[0]);
      stage_b(f, U2, U, 0.5, U1, 0.5, 0.5 * dt);
      convergence(f, U1, U2);
      if (!subcycle_check(f)) break;
      dt = dt / 10.0;
    }
    for (int k = 0; k < 4; ++k) memcpy(U[k], U2[k], nfield(d) * sizeof(double));
  } else if (f->c.rk == CATO_RK_SSP3) {
    double* U1[4] = {f->st[0][0], f->st[0][1], f->st[0][2], f->st[0][3]};
    double* U2[4] = {f->st[1][0], f->st[1][1], f->st[1][2], f->st[1][3]};
    double* U3[4] = {f->st[2][0], f->st[2][1], f->st[2][2], f->st[2][3]};
    for (;;) {  /* ssp_rk_3_3's subcycle loop, mod_fluid.f90:762-829 */
      f->solver_time = f->solver_time + dt;
      f->bc_time = f->solver_time;
      rc |= residual(f, f->rho, f->u, f->v, f->p);
      stage_a(f, U1, U, dt);
      derive_all(f, U1, su[0], sv[0], spp[0], scs[0]);
      f->bc_time = f->time + dt;
      rc |= residual(f, U1[0], su[0], sv[0], spp[0]);
      stage_b(f, U2, U, 3.0 / 4.0, U1, 1.0 / 4.0, (1.0 / 4.0) * dt);
      derive_all(f, U2, su[1], sv[1], spp[1], scs[1]);
      rc |= residual(f, U2[0], su[1], sv[1], spp[1]);
      stage_b(f, U3, U, 1.0 / 3.0, U2, 2.0 / 3.0, (2.0 / 3.0) * dt);
      convergence(f, U1, U3);
      if (!subcycle_check(f)) break;
      dt = dt / 10.0;
    }
    for (int k = 0; k < 4; ++k) memcpy(U[k], U3[k], nfield(d) * sizeof(double));
  } else {
    /* rk(m,n), mod_fluid.f90:926-966 */
    static const double a13[] = {0.1481, 0.4, 1.0}, a14[] = {0.0833, 0.2069, 0.4265, 1.0},
                        a15[] = {0.0533, 0.1263, 0.2375, 0.4414, 1.0}, a23[] = {0.1918, 0.4929, 1.0},
                        a24[] = {0.1084, 0.2602, 0.5052, 1.0},
                        a25[] = {0.0695, 0.1602, 0.2898, 0.5060, 1.0};
    const double* alpha;
    int ns;
    switch (f->c.rk) {
      case CATO_RK_1_3: alpha = a13; ns = 3; break;
      case CATO_RK_1_4: alpha = a14; ns = 4; break;
      case CATO_RK_1_5: alpha = a15; ns = 5; break;
      case CATO_RK_2_3: alpha = a23; ns = 3; break;
      case CATO_RK_2_4: alpha = a24; ns = 4; break;
      default: alpha = a25; ns = 5; break;
    }
    double* U0[4] = {f->st[0][0], f->st[0][1], f->st[0][2], f->st[0][3]};
    double* Uc[4] = {f->st[1][0], f->st[1][1], f->st[1][2], f->st[1][3]};
    for (int k = 0; k < 4; ++k) memcpy(U0[k], U[k], nfield(d) * sizeof(double));
    /* U_prev starts as a copy of U (its primitives are U's) */
    for (int m = 0; m < ns; ++m) {
      /* m = 1: U_prev is a fresh copy of U (allocate(source=U)) and carries U's solver clock,
       * which rk_multistage never advances; later U_prev = U_curr restarts it at U%time */
      f->bc_time = (m == 0) ? f->solver_time + dt : t_copy;
      if (m == 0) rc |= residual(f, f->rho, f->u, f->v, f->p);
      else rc |= residual(f, Uc[0], su[0], sv[0], spp[0]);
      stage_a(f, Uc, U0, dt * alpha[m]);
      derive_all(f, Uc, su[0], sv[0], spp[0], scs[0]);
    }
    convergence(f, U0, Uc);
    for (int k = 0; k < 4; ++k) memcpy(U[k], Uc[k], nfield(d) * sizeof(double));
  }
  f->dt = dt;
  f->time = f->time + dt;
  derive_all(f, U, f->u, f->v, f->p, f->cs);
  /* the reference's order of checks: check_for_nans on rho, u, v, p at the stage assignment
   * (assign_fluid, mod_fluid.f90:718-721; field_2d.f90:825-844), then sanity_check's negative
   * density, then negative pressure over the whole field (mod_fluid.f90:726-737;
   * field_2d.f90:846-867); the first failing check stops (error.f90:6-9 codes) */
  int32_t ec = 0;
  for (int j = 1; j <= d.nj && !ec; ++j)
    for (int i = 1; i <= d.ni && !ec; ++i)
      if (isnan(AT(f->rho, i, j)) || isnan(AT(f->u, i, j)) || isnan(AT(f->v, i, j)) ||
          isnan(AT(f->p, i, j)))
        ec = CATO_NANS_FOUND;
  for (int j = 1; j <= d.nj && !ec; ++j)
    for (int i = 1; i <= d.ni && !ec; ++i)
      if (AT(f->rho, i, j) < 0.0) ec = CATO_NEG_DENSITY;
  for (int j = 1; j <= d.nj && !ec; ++j)
    for (int i = 1; i <= d.ni && !ec; ++i)
      if (AT(f->p, i, j) < 0.0) ec = CATO_NEG_PRESSURE;
  if (error_code) *error_code = ec;
  for (int s = 0; s < 4; ++s) { free(su[s]); free(sv[s]); free(spp[s]); free(scs[s]); }
  return rc;
}

int oracle_get_state(oracle_fluid* f, double* rho, double* rho_u, double* rho_v, double* rho_E,
                     double* u, double* v, double* p, double* cs) {
  size_t n = nfield(f->d) * sizeof(double);
  dims_t d = f->d;
  double* src[8] = {f->rho, f->rhou, f->rhov, f->rhoE, f->u, f->v, f->p, f->cs};
  double* dst[8] = {rho, rho_u, rho_v, rho_E, u, v, p, cs};
  for (int k = 0; k < 8; ++k) {
    if (!dst[k]) continue;
    memset(dst[k], 0, n);
    for (int j = 1; j <= d.nj; ++j)
      for (int i = 1; i <= d.ni; ++i) AT(dst[k], i, j) = AT(src[k], i, j);
  }
  return 0;
}

double oracle_time(oracle_fluid* f) { return f->time; }
int64_t oracle_iteration(oracle_fluid* f) { return f->iteration; }

/* ------------------------------------------------------------------------------------------ */
/* configuration                                                                                */
/* ------------------------------------------------------------------------------------------ */
int oracle_config_default(cato_config* c, int32_t ni, int32_t nj) {
  if (!c) return CATO_ERR_ARG;
  memset(c, 0, sizeof(*c));
  c->ni = ni;
  c->nj = nj;
  c->n_ghost = 2;
  c->flux = CATO_FLUX_AUSMPW_PLUS;
  c->limiter = CATO_LIM_MINMOD;
  c->rk = CATO_RK_SSP2;
  for (int s = 0; s < 4; ++s) c->bc[s] = CATO_BC_PERIODIC;
  c->apply_low_mach_fix = 1;
  c->precision = CATO_FP64;
  c->roe_entropy_fix = CATO_ROE_REFERENCE;
  c->gamma = 5.0 / 3.0;
  c->cfl = 0.1;
  c->dx = 1.0;
  c->dy = 1.0;
  c->harten_delta = 0.1;
  c->ausm_beta = 1.0 / 8.0;
  c->ausm_kp = 0.25;
  c->ausm_ku = 0.75;
  c->ausm_sigma = 1.0;
  return CATO_OK;
}

int oracle_config_check(const cato_config* c) {
  if (!c) return CATO_ERR_ARG;
  if (c->ni < 1 || c->nj < 1) return CATO_ERR_CONFIG;
  if (c->flux < CATO_FLUX_AUSMPW_PLUS || c->flux > CATO_FLUX_M_AUSMPW_PLUS) return CATO_ERR_CONFIG;
  if (c->limiter < CATO_LIM_MINMOD || c->limiter > CATO_LIM_MLP5) return CATO_ERR_CONFIG;
  if (c->rk < CATO_RK_SSP2 || c->rk > CATO_RK_2_5) return CATO_ERR_CONFIG;
  int need = (c->limiter == CATO_LIM_MLP5) ? 3 : 2; /* mod_input.f90:320-338 */
  if (c->n_ghost != need) return CATO_ERR_CONFIG;
  if (c->ni < c->n_ghost || c->nj < c->n_ghost) return CATO_ERR_CONFIG;
  int outlet = 0, exchange = 0, pinput = 0;
  for (int s = 0; s < 4; ++s) {
    if (c->bc[s] < CATO_BC_ZERO_GRADIENT || c->bc[s] > CATO_BC_EXCHANGE) return CATO_ERR_CONFIG;
    /* the pressure input only implements +x (pressure_input_bc.f90:404-409) */
    if (c->bc[s] == CATO_BC_PRESSURE_INPUT && s != CATO_PLUS_X) return CATO_ERR_CONFIG;
    outlet |= c->bc[s] == CATO_BC_OUTLET;
    pinput |= c->bc[s] == CATO_BC_PRESSURE_INPUT;
    /* slab cuts are rows: +-y only */
    if (c->bc[s] == CATO_BC_EXCHANGE && s != CATO_PLUS_Y && s != CATO_MINUS_Y)
      return CATO_ERR_CONFIG;
    exchange |= c->bc[s] == CATO_BC_EXCHANGE;
  }
  if (exchange && pinput) return CATO_ERR_CONFIG;
  if (outlet && !(c->bc_pressure > 0.0)) return CATO_ERR_CONFIG; /* outlet_bc.f90:54-59 */
  /* periodic must be paired on an axis (an unpaired side leaves ghost cells unset) */
  if ((c->bc[CATO_PLUS_X] == CATO_BC_PERIODIC) != (c->bc[CATO_MINUS_X] == CATO_BC_PERIODIC))
    return CATO_ERR_CONFIG;
  if ((c->bc[CATO_PLUS_Y] == CATO_BC_PERIODIC) != (c->bc[CATO_MINUS_Y] == CATO_BC_PERIODIC))
    return CATO_ERR_CONFIG;
  if (!(c->gamma > 1.0) || !(c->cfl > 0.0) || !(c->dx > 0.0) || !(c->dy > 0.0))
    return CATO_ERR_CONFIG;
  /* the oracle computes in FP64 whatever the precision asks of the GPU path */
  if (c->precision < CATO_FP64 || c->precision > CATO_MIXED_DF) return CATO_ERR_CONFIG;
  if (c->roe_entropy_fix != CATO_ROE_REFERENCE && c->roe_entropy_fix != CATO_ROE_HARTEN)
    return CATO_ERR_CONFIG;
  return CATO_OK;
}
