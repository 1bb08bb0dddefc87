// cato_kernels.cuh -- small kernels around the stage kernel: upload (primitive -> conserved with
// the initial CFL dt), per-step control, derived-quantity download, ghost fill and the
// stand-alone edge reconstruction.  Built with --fmad=false (FP64 reference arithmetic).
#pragma once

#include "cato_ctl.cuh"
#include "cato_stage.cuh"

namespace cato {

// one thread: decide whether this step runs and with which dt (master_puppeteer.f90:155-200)
static __global__ void step_begin_kernel(StepCtl* c) {
  int act = (c->status == 0) && (c->time < c->t_end) && (c->iter < c->max_iter);
  c->active = act;
  if (!act) return;
  double dt = c->fixed_dt > 0.0 ? c->fixed_dt : decode_dt(c->dt_min);
  c->dt = dt;
  c->t_step = c->time;
  c->time = c->time + dt;
  c->iter = c->iter + 1;
  c->dt_min = ~0ULL;
}

// initialize_from_hdf5 + eos%primitive_to_conserved (equation_of_state.f90:316-324 through the
// field operators) and the CFL dt of the raw primitives (mod_fluid.f90:249, 518-562).
static __global__ void upload_init_kernel(int ni, int nj, int pitch, double gamma, double cfl, double dx,
                                   double dy, const double* __restrict__ dxc,
                                   const double* __restrict__ dyc, const double* __restrict__ r_,
                                   const double* __restrict__ u_, const double* __restrict__ v_,
                                   const double* __restrict__ p_, double* rho, double* rhou,
                                   double* rhov, double* rhoE, StepCtl* ctl) {
  const double EPS = Num<double>::eps, TINY = Num<double>::tiny;
  const double g1 = gamma - 1.0, one_over_g1 = 1.0 / g1;
  double dmin = INFINITY;
  int st = 0;
  // rows of the grid-stride loop: a 32-bit index split while the grid has fewer than 2^32 cells
  // (a 64-bit integer division per cell costs more than the rest of the cell's work)
  const long long total = (long long)ni * nj;
  const bool narrow = total <= 0xffffffffLL;
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < total;
       n += (long long)gridDim.x * blockDim.x) {
    int i, j;
    if (narrow) {
      j = (int)((unsigned)n / (unsigned)ni);
      i = (int)((unsigned)n - (unsigned)j * (unsigned)ni);
    } else {
      j = (int)(n / ni);
      i = (int)(n - (long long)j * ni);
    }
    const size_t idx = (size_t)j * pitch + i;
    const double r = r_[idx], u = u_[idx], v = v_[idx], p = p_[idx];
    rho[idx] = r;
    rhou[idx] = u * r;
    rhov[idx] = v * r;
    double s = u * u + v * v;
    if (abs_lt(s, EPS)) s = 0.0;
    double E = p * one_over_g1 + (r * 0.5) * s;
    if (abs_lt(E, EPS)) E = 0.0;
    rhoE[idx] = E;
    // the divisions and the square root on the integer pipe (correctly rounded, so the values
    // equal the FP64 instructions')
    const double pr = abs_lt(p, TINY) ? 0.0 : div_rn(p, r);
    const double cs = sqrt_rn(gamma * pr);
    // min_dx / min_dy of the cell: per column / row on a rectilinear grid
    const double cdx = dxc ? dxc[i] : dx, cdy = dyc ? dyc[j] : dy;
    const double d = div_rn(cfl, div_rn(fabs(u) + cs, cdx) + div_rn(fabs(v) + cs, cdy));
    if (d < dmin) dmin = d;
    if (isnan(r) || isnan(u) || isnan(v) || isnan(p)) st |= ST_NAN;
    // initialize_from_hdf5 refuses ~0 density or pressure (mod_fluid.f90:352-360)
    if (r < TINY) st |= ST_NEG_DENSITY;
    if (p < TINY) st |= ST_NEG_PRESSURE;
  }
  unsigned long long bits = (dmin > 0.0) ? (unsigned long long)__double_as_longlong(dmin) : ~0ULL;
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long ob = __shfl_xor_sync(0xffffffffu, bits, o);
    bits = ob < bits ? ob : bits;
    st |= __shfl_xor_sync(0xffffffffu, st, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (bits != ~0ULL) atomicMin(&ctl->dt_min, bits);
    if (st) atomicOr(&ctl->status, st);
  }
}

// fluid_t's derived quantities for download: u, v, p, cs of the conserved state (FP64,
// calculate_derived_quantities), or of the raw primitives before the first step.
static __global__ void derive_kernel(int ni, int nj, int pitch, double gamma, int raw,
                              const double* __restrict__ a0, const double* __restrict__ a1,
                              const double* __restrict__ a2, const double* __restrict__ a3,
                              double* u, double* v, double* p, double* cs) {
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < (long long)ni * nj;
       n += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(n % ni), j = (int)(n / ni);
    const size_t idx = (size_t)j * pitch + i;
    if (raw) {
      const double r = a0[idx], pp = a3[idx];
      u[idx] = a1[idx];
      v[idx] = a2[idx];
      p[idx] = pp;
      const double pr = abs_lt(pp, Num<double>::tiny) ? 0.0 : pp / r;
      cs[idx] = sqrt(gamma * pr);
    } else {
      double uu, vv, pp, cc;
      prim_from_cons(gamma, gamma - 1.0, a0[idx], a1[idx], a2[idx], a3[idx], uu, vv, pp, cc);
      u[idx] = uu;
      v[idx] = vv;
      p[idx] = pp;
      cs[idx] = cc;
    }
  }
}

// Halo-padded primitive fields with every ghost cell filled by the boundary conditions, as after
// flux_solver_t%apply_primitive_bc (flux_solver.f90:138-185).
static __global__ void fill_ghosts_kernel(int ni, int nj, int pitch, int ng, int4 bc,
                                   double gamma, double bc_p, const double* __restrict__ pbc_edge,
                                   const double* __restrict__ r_, const double* __restrict__ u_,
                                   const double* __restrict__ v_, const double* __restrict__ p_,
                                   double* ro, double* uo, double* vo, double* po, long long ld) {
  const int W = ni + 2 * ng, H = nj + 2 * ng;
  const int bcs[4] = {bc.x, bc.y, bc.z, bc.w};
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < (long long)W * H;
       n += (long long)gridDim.x * blockDim.x) {
    const int ii = (int)(n % W), jj = (int)(n / W);
    bool fx, fy;
    const int sx = map_index(ii - ng, ni, bcs[SIDE_MX], bcs[SIDE_PX], fx);
    const int sy = map_index(jj - ng, nj, bcs[SIDE_MY], bcs[SIDE_PY], fy);
    const size_t s = (size_t)sy * pitch + sx;
    const size_t o = (size_t)jj * ld + ii;
    double r = r_[s], u = fx ? -u_[s] : u_[s], v = fy ? -v_[s] : v_[s], p = p_[s];
    if (bcs[SIDE_PX] == BC_OUTLET && ii - ng >= ni) outlet_ghost<double>(gamma, bc_p, r, u, v, p);
    if (bcs[SIDE_PX] == BC_PRESSURE_INPUT && ii - ng >= ni) {  // the row's edge state
      const double* e = pbc_edge + 3 * (size_t)jj;
      r = e[0];
      u = e[1];
      v = 0.0;
      p = e[2];
    }
    ro[o] = r;
    uo[o] = u;
    vo[o] = v;
    po[o] = p;
  }
}

// muscl_interpolation_t%interpolate_edge_values on a halo-filled field q (ld = ni + 2 ng):
// i_edges(1:2, -1:ni, 0:nj) and j_edges(1:2, 0:ni, -1:nj), both computed for i, j = 0..ni, 0..nj.
template <int NG, int RECON>
static __global__ void interp_edges_kernel(int ni, int nj, int lim, const double* __restrict__ q,
                                    long long ld, double* ie, double* je) {
  auto Q = [&](int i, int j) -> double {  // reference (i, j), 1-based interior
    return q[(size_t)(j + NG - 1) * ld + (i + NG - 1)];
  };
  const long long n_e = (long long)(ni + 1) * (nj + 1);
  for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < n_e;
       n += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(n % (ni + 1)), j = (int)(n / (ni + 1));
    double L, R;
    // i-direction edge (i+1/2, j)
    if (RECON == 0) {
      recon_tvd2<double>(lim, Q(i - 1, j), Q(i, j), Q(i + 1, j), Q(i + 2, j), L, R);
    } else {
      recon_mlp<double, RECON>(RECON == 5 ? Q(i - 2, j) : 0.0, Q(i - 1, j), Q(i, j), Q(i + 1, j),
                               Q(i + 2, j), RECON == 5 ? Q(i + 3, j) : 0.0, Q(i, j + 1),
                               Q(i, j - 1), Q(i + 1, j + 1), Q(i + 1, j - 1), L, R);
    }
    const size_t oi = 2 * ((size_t)(i + 1) + (size_t)j * (ni + 2));
    ie[oi] = L;
    ie[oi + 1] = R;
    // j-direction edge (i, j+1/2)
    if (RECON == 0) {
      recon_tvd2<double>(lim, Q(i, j - 1), Q(i, j), Q(i, j + 1), Q(i, j + 2), L, R);
    } else {
      recon_mlp<double, RECON>(RECON == 5 ? Q(i, j - 2) : 0.0, Q(i, j - 1), Q(i, j), Q(i, j + 1),
                               Q(i, j + 2), RECON == 5 ? Q(i, j + 3) : 0.0, Q(i + 1, j),
                               Q(i - 1, j), Q(i + 1, j + 1), Q(i - 1, j + 1), L, R);
    }
    const size_t oj = 2 * ((size_t)i + (size_t)(j + 1) * (ni + 1));
    je[oj] = L;
    je[oj + 1] = R;
  }
}

// Deterministic FP64 reductions over the interior: a fixed partition (block b takes rows
// b, b + RED_BLOCKS, ...; thread t takes columns t, t + RED_THREADS, ...) and a fixed summation
// tree, so a result depends only on the data and the grid size, never on scheduling.
constexpr int RED_BLOCKS = 304;  // 2 x 152 SMs
constexpr int RED_THREADS = 256;
constexpr int RED_Q = 8;         // quantities per reduction

struct RedArgs {
  int ni, nj, pitch;
  int mode;               // 0: sums of A; 1: sums of (B - A)^2 and A^2
  const double* A[4];
  const double* B[4];
  const double* dxc;      // mode 0 on a rectilinear grid: the sums are of A * dx_i * dy_j
  const double* dyc;
  double* partials;       // RED_BLOCKS x RED_Q
};

__device__ __forceinline__ double block_sum(double x, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = x;
  __syncthreads();
  x = (threadIdx.x < (RED_THREADS >> 5)) ? sh[threadIdx.x] : 0.0;
  if (w == 0) {
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  }
  return x;  // valid in thread 0
}

static __global__ void __launch_bounds__(RED_THREADS) reduce_partials_kernel(RedArgs R) {
  __shared__ double sh[RED_THREADS / 32];
  double acc[RED_Q];
#pragma unroll
  for (int q = 0; q < RED_Q; ++q) acc[q] = 0.0;
  for (int j = blockIdx.x; j < R.nj; j += gridDim.x) {
    for (int i = threadIdx.x; i < R.ni; i += blockDim.x) {
      const size_t idx = (size_t)j * R.pitch + i;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        double a = R.A[k][idx];
        if (R.mode == 0) {
          acc[k] += R.dxc ? a * (R.dxc[i] * R.dyc[j] - 0.0 * 0.0) : a;
        } else {
          const double df = R.B[k][idx] - a;
          acc[k] += df * df;
          acc[4 + k] += a * a;
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < RED_Q; ++q) {
    const double s = block_sum(acc[q], sh);
    if (threadIdx.x == 0) R.partials[blockIdx.x * RED_Q + q] = s;
  }
}

// one block: out[q] = sum over blocks of partials[b][q], in a fixed order
static __global__ void __launch_bounds__(RED_THREADS) reduce_final_kernel(const double* partials,
                                                                          int n_blocks,
                                                                          double* out) {
  __shared__ double sh[RED_THREADS / 32];
  for (int q = 0; q < RED_Q; ++q) {
    double x = 0.0;
    for (int b = threadIdx.x; b < n_blocks; b += blockDim.x) x += partials[b * RED_Q + q];
    x = block_sum(x, sh);
    if (threadIdx.x == 0) out[q] = x;
  }
}

}  // namespace cato
