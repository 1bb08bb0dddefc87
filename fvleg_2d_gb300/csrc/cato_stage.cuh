// cato_stage.cuh -- the fused RK stage kernel: ghost-cell boundary conditions, primitive
// recovery, MUSCL/MLP reconstruction, edge fluxes, flux divergence and the RK stage combine in
// one pass over HBM, with the CFL dt min-reduction and the state checks fused into the last stage.
//
// Work decomposition ("marching strip"): a CTA of T threads owns a strip of W = T - 2*NG output
// columns and marches over rows_per_cta rows.  Thread t always handles column x0 - NG + t, so a
// row of primitives (T cells incl. the x-halo) is produced by one coalesced row load.  Shared
// memory keeps a ring of the last 2*NG primitive rows, the i-edge fluxes of the current row and
// the j-edge fluxes below/above it; each row costs two __syncthreads.  Every primitive is
// computed once per stage (x-halo overhead 2*NG/T, y-halo 2*NG/rows_per_cta).
//
// Ghost cells are never stored: a ghost row/column index maps to its source interior cell
// (zero-gradient copy, symmetry mirror with the normal velocity negated, periodic wrap).  This
// reproduces the reference's sequential application (flux_solver.f90:138-185, zero_gradient
// full-length rows incl. corners, periodic corners only when all four sides are periodic)
// because for every valid side combination the final ghost value is that composition.
#pragma once

#include "cato_physics.cuh"

namespace cato {

// How a compute type computes a stage.  Every precision keeps the same structure-of-arrays FP64
// state and FP64 stage buffers, and combines the stages (the RK accumulation) in FP64.
//   0 FP64    : reconstruction, flux and divergence in FP64 (bit-exact drop-in path)
//   1 FP32    : the stencil's conserved values rounded to FP32; reconstruction, flux and
//               divergence in FP32 (mixed)
//   2 df      : reconstruction, flux and divergence in double-float (mixed_df)
template <typename R> struct Prec;
template <> struct Prec<double> { static constexpr int kind = 0; };
template <> struct Prec<float> { static constexpr int kind = 1; };
template <> struct Prec<df> { static constexpr int kind = 2; };

struct StageArgs {
  int ni, nj, pitch;       // interior cells, row pitch (cells) of the state arrays
  int bc[4];               // by side: +x, +y, -x, -y
  int limiter;             // TVD2 limiter id (runtime)
  int rows_per_cta;
  int kind;                // 0: out = U_a + L*c ; 1: out = (U_a*a + U_k*b) + L*c  (each '+'
                           // flushed) ; 2: out = L (flux_solver_t%solve output, FP64 path)
  int last;                // last stage of the step: emit the CFL dt and the state checks
  double a, b, coef;       // c = coef * dt (the reference's (0.5_rk*dt), ((1/4)*dt), dt*alpha ...)
  // structure of arrays, one FP64 array per conserved variable
  const double* Uk[4];     // conserved state of this stage (stencil operand)
  const double* Ua[4];     // U_a (point-wise operand; the step's U^n)
  double* Uo[4];           // output conserved state
  const double* Pin[4];    // when non-null: primitives to use as-is for this stage (after upload)
  // device scalars
  const double* dt;
  const int* active;
  unsigned long long* dt_min;  // bits of the smallest positive dt candidate (atomicMin)
  int* status;
  // physics
  double gamma, cfl;
  double bc_p;             // outlet pressure (CATO_BC_OUTLET)
  // +x pressure input (CATO_BC_PRESSURE_INPUT): the ghost state (rho, u, p; v = 0) of rows
  // -pbc_ng .. nj+pbc_ng-1, written for this stage by pbc_edge_kernel
  const double* pbc_edge;
  int pbc_ng;
  // energy source term: q_dot_h per interior cell (pitch layout), added to the energy residual
  // (time_derivative, mod_fluid.f90:503); null without a source
  const double* src_q;
  Geom G;
};

// Source interior index of (possibly ghost) index g in [-ng, n+ng) along an axis with
// boundary types lo/hi; flip = the normal velocity component is negated (symmetry).  An
// exchange side (the rows axis of a slab only) keeps g: its ghost rows are stored below row 0
// and above row n - 1 of the slab's buffers, copied from the neighbouring slab.
__device__ __forceinline__ int map_index(int g, int n, int bc_lo, int bc_hi, bool& flip) {
  flip = false;
  if (g < 0) {
    if (bc_lo == BC_PERIODIC) return max(n + g, 0);
    if (bc_lo == BC_SYMMETRY) { flip = true; return min(-g - 1, n - 1); }
    if (bc_lo == BC_EXCHANGE) return g;
    return 0;
  }
  if (g >= n) {
    if (bc_hi == BC_PERIODIC) return min(g - n, n - 1);
    if (bc_hi == BC_SYMMETRY) { flip = true; return max(2 * n - 1 - g, 0); }
    if (bc_hi == BC_EXCHANGE) return g;
    return n - 1;
  }
  return g;
}

// Outlet ghost state on the +x side (outlet_bc.f90:101-123) from the primitives of the boundary
// cell it maps to (after the other sides' BCs, as the outlet has the lowest priority): copied
// when the boundary cell is supersonic, else the characteristic subsonic outflow state at the
// ambient pressure p_b.  The reference leaves the ghost unchanged when p_b or the boundary
// density is below tiny (p_b > 0 is enforced by the configuration check); here it keeps the copy.
template <typename R>
__device__ __forceinline__ void outlet_ghost(R gamma, R p_b, R& r, R& u, R& v, R& p) {
  const R r0 = r, p_d = p;
  if (!(p_b > Num<R>::tiny) || !(r0 > Num<R>::tiny)) return;
  const R cs = Num<R>::sqrt(gamma * rabs(Num<R>::div(p_d, r0)));
  const R vel = Num<R>::sqrt(u * u + v * v);
  const R mach = Num<R>::div(vel, cs);
  const R nx = Num<R>::div(u, vel + R(1e-30));
  const R ny = Num<R>::div(v, vel + R(1e-30));
  if (mach > R(1)) return;
  r = r0 + Num<R>::div(p_b - p_d, cs * cs);
  u = u + Num<R>::div(nx * (p_d - p_b), r0 * cs);
  v = v + Num<R>::div(ny * (p_d - p_b), r0 * cs);
  p = p_b;
}

template <int RING> __device__ __forceinline__ int slot_of(int row) {
  return (row + 4 * RING) % RING;  // rows are >= -NG
}

// Row bases of the shared-memory ring for rows center-2 .. center+3 (each row: [var][col]).
template <typename R, int RING>
__device__ __forceinline__ void ring_rows(R* ring, int T, int center, const R* rp[6]) {
#pragma unroll
  for (int k = 0; k < 6; ++k) rp[k] = ring + slot_of<RING>(center + k - 2) * 4 * T;
}

// ---------------------------------------------------------------------------------------------
// one edge: reconstruct the four primitives from the ring and evaluate the flux
// ---------------------------------------------------------------------------------------------
template <typename R, int NG, int FLUX, int RECON, int DIR>
__device__ __forceinline__ void edge_flux(const R* const rp[6], int T, int lim, int col,
                                          const FluxConsts<R>& K, R F[4]) {
  // stencil sample at normal offset n and tangential offset t from the edge's left cell;
  // rp[k] is the ring row (edge row) + k - 2
  auto Q = [&](int var, int n, int t) -> R {
    return DIR == 0 ? rp[t + 2][var * T + col + n] : rp[n + 2][var * T + col + t];
  };
  R Lv[4], Rv[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (RECON == 0) {
      if constexpr (Prec<R>::kind == 0) {
        const EdgePair e = recon_tvd2_f64(lim, Q(k, -1, 0), Q(k, 0, 0), Q(k, 1, 0), Q(k, 2, 0));
        Lv[k] = e.L;
        Rv[k] = e.R;
      } else {
        recon_tvd2<R>(lim, Q(k, -1, 0), Q(k, 0, 0), Q(k, 1, 0), Q(k, 2, 0), Lv[k], Rv[k]);
      }
    } else {
      R qm2 = RECON == 5 ? Q(k, -2, 0) : R(0), qp3 = RECON == 5 ? Q(k, 3, 0) : R(0);
      if constexpr (Prec<R>::kind == 0) {
        const EdgePair e = recon_mlp_f64<RECON>(qm2, Q(k, -1, 0), Q(k, 0, 0), Q(k, 1, 0),
                                                Q(k, 2, 0), qp3, Q(k, 0, 1), Q(k, 0, -1),
                                                Q(k, 1, 1), Q(k, 1, -1));
        Lv[k] = e.L;
        Rv[k] = e.R;
      } else {
        recon_mlp<R, RECON>(qm2, Q(k, -1, 0), Q(k, 0, 0), Q(k, 1, 0), Q(k, 2, 0), qp3,
                            Q(k, 0, 1), Q(k, 0, -1), Q(k, 1, 1), Q(k, 1, -1), Lv[k], Rv[k]);
      }
    }
  }
  Prim<R> A = {Lv[0], Lv[1], Lv[2], Lv[3]}, B = {Rv[0], Rv[1], Rv[2], Rv[3]};
  // cell pressures in reference (i, j) terms: P(di, dj) = p(i+di, j+dj), (i, j) = left cell
  auto P = [&](int di, int dj) -> R { return DIR == 0 ? Q(3, di, dj) : Q(3, dj, di); };
  if (FLUX == FLUX_AUSMPW || FLUX == FLUX_M_AUSMPW) {
    R pc[4];
    if (DIR == 0) { pc[0] = P(0, -1); pc[1] = P(1, -1); pc[2] = P(0, 1); pc[3] = P(1, 1); }
    else { pc[0] = P(1, 0); pc[1] = P(1, 1); pc[2] = P(-1, 0); pc[3] = P(-1, 1); }
    if constexpr (FLUX == FLUX_M_AUSMPW) {
      // the superbee edge states of the second interpolator (m_ausmpw_plus_solver.fypp:163-167)
      R Ls[4], Rs[4];
#pragma unroll
      for (int k = 0; k < 4; ++k)
        recon_tvd2<R>(LIM_SUPERBEE, Q(k, -1, 0), Q(k, 0, 0), Q(k, 1, 0), Q(k, 2, 0), Ls[k], Rs[k]);
      Prim<R> As = {Ls[0], Ls[1], Ls[2], Ls[3]}, Bs = {Rs[0], Rs[1], Rs[2], Rs[3]};
      flux_mausmpw<R, DIR>(K, A, B, As, Bs, pc, F);
    } else {
      flux_ausmpw<R, DIR>(K, A, B, pc, F);
    }
  } else if (FLUX == FLUX_SLAU || FLUX == FLUX_SLAU2 || FLUX == FLUX_SD_SLAU ||
             FLUX == FLUX_SD_SLAU2) {
    R pa[6], pb[6];
    if (FLUX == FLUX_SD_SLAU || FLUX == FLUX_SD_SLAU2) {
      if (DIR == 0) {  // slau_solver.fypp:410-417
        pa[0] = P(0, 1);  pb[0] = P(0, 0);
        pa[1] = P(-1, 0); pb[1] = P(0, 0);
        pa[2] = P(0, -1); pb[2] = P(0, 0);
        pa[3] = P(1, -1); pb[3] = P(1, 0);
        pa[4] = P(2, 0);  pb[4] = P(1, 0);
        pa[5] = P(1, 1);  pb[5] = P(1, 0);
      } else {         // slau_solver.fypp:421-428
        pa[0] = P(-1, 0); pb[0] = P(0, 0);
        pa[1] = P(0, -1); pb[1] = P(0, 0);
        pa[2] = P(1, 0);  pb[2] = P(0, 0);
        pa[3] = P(1, 1);  pb[3] = P(0, 1);
        pa[4] = P(0, 2);  pb[4] = P(0, 1);
        pa[5] = P(-1, 1); pb[5] = P(0, 1);
      }
    }
    flux_slau<R, DIR, FLUX>(K, A, B, pa, pb, F);
  } else if (FLUX == FLUX_ROE) {
    R fa[5], fb[5];
    if (DIR == 0) {  // roe_solver.fypp:496-500
      fa[0] = P(0, 0); fb[0] = P(1, 0);
      fa[1] = P(0, 0); fb[1] = P(0, 1);
      fa[2] = P(0, 0); fb[2] = P(0, -1);
      fa[3] = P(0, 1); fb[3] = P(1, 1);
      fa[4] = P(0, -1); fb[4] = P(1, -1);
    } else {         // roe_solver.fypp:502-506
      fa[0] = P(0, 0); fb[0] = P(0, 1);
      fa[1] = P(0, 0); fb[1] = P(-1, 0);
      fa[2] = P(0, 0); fb[2] = P(1, 0);
      fa[3] = P(0, 1); fb[3] = P(-1, 1);
      fa[4] = P(0, 1); fb[4] = P(1, 1);
    }
    flux_roe<R, DIR>(K, A, B, fa, fb, F);
  } else if (FLUX == FLUX_AUSM_UP) {
    flux_ausm_up<R, DIR>(K, A, B, F);
  } else {
    flux_hllc<R, DIR>(K, A, B, F);
  }
}

// ---------------------------------------------------------------------------------------------
// primitive row load
// ---------------------------------------------------------------------------------------------
template <typename R> struct RowSrc {
  double c[4];  // conserved state of the stage (or the raw primitives) as loaded
  bool flipy;
};

template <typename R>
__device__ __forceinline__ void load_src(const StageArgs& A, int sx, int row, RowSrc<R>& s) {
  bool fy;
  const int sy = map_index(row, A.nj, A.bc[SIDE_MY], A.bc[SIDE_PY], fy);
  s.flipy = fy;
  const size_t idx = (size_t)sy * A.pitch + sx;
  const double* const* src = A.Pin[0] ? A.Pin : A.Uk;
#pragma unroll
  for (int k = 0; k < 4; ++k) s.c[k] = __ldg(src[k] + idx);
}

template <typename R> __device__ __forceinline__ R from_double(double x);
template <> __device__ __forceinline__ double from_double<double>(double x) { return x; }
template <> __device__ __forceinline__ float from_double<float>(double x) { return d2f_int(x); }
template <> __device__ __forceinline__ df from_double<df>(double x) { return to_df(x); }

// xmode: 0 interior / mapped ghost, 1 +x outlet ghost column, 2 +x pressure-input ghost column;
// row: the (possibly ghost) row of the sample
template <typename R>
__device__ __forceinline__ void src_to_prim(const StageArgs& A, const RowSrc<R>& s, bool flipx,
                                            int xmode, int row, R g, R g1, R out[4]) {
  if (xmode == 2) {  // lowest-priority BC: the row's edge state replaces the mapped value
    const double* e = A.pbc_edge + 3 * (size_t)(row + A.pbc_ng);
    out[0] = from_double<R>(e[0]);
    out[1] = from_double<R>(e[1]);
    out[2] = R(0);
    out[3] = from_double<R>(e[2]);
    return;
  }
  R r, u, v, p;
  if constexpr (Prec<R>::kind == 0) {
    if (A.Pin[0]) {
      r = s.c[0]; u = s.c[1]; v = s.c[2]; p = s.c[3];
    } else {
      R cs;
      r = s.c[0];
      prim_from_cons(g, g1, r, s.c[1], s.c[2], s.c[3], u, v, p, cs);
    }
  } else if constexpr (Prec<R>::kind == 2) {
    if (A.Pin[0]) {
      r = to_df(s.c[0]); u = to_df(s.c[1]); v = to_df(s.c[2]); p = to_df(s.c[3]);
    } else {
      R cs;
      r = to_df(s.c[0]);
      const df rE = to_df(s.c[3]);
      prim_from_cons(g, g1, r, to_df(s.c[1]), to_df(s.c[2]), rE, u, v, p, cs, false);
      if (near_vacuum(p.hi, rE.hi, 1e-4f)) {
        double u64, v64, p64;
        prim_from_cons_f64(A.gamma, s.c[0], s.c[1], s.c[2], s.c[3], u64, v64, p64);
        u = to_df(u64); v = to_df(v64); p = to_df(p64);
      }
    }
  } else {
    r = d2f_fast(s.c[0]);
    if (A.Pin[0]) {
      u = d2f_fast(s.c[1]); v = d2f_fast(s.c[2]); p = d2f_fast(s.c[3]);
    } else {
      R cs;
      prim_from_cons(g, g1, r, d2f_fast(s.c[1]), d2f_fast(s.c[2]), d2f_fast(s.c[3]), u, v, p,
                     cs);
    }
  }
  u = flipx ? -u : u;
  v = s.flipy ? -v : v;
  if (xmode == 1) outlet_ghost<R>(g, R(A.bc_p), r, u, v, p);
  out[0] = r;
  out[1] = u;
  out[2] = v;
  out[3] = p;
}

// ---------------------------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------------------------
// One tile: columns [bx*W, bx*W + W) x rows [by*rows_per_cta, ...) of one instance.
// EXT = false compiles out the rectilinear metrics, the energy source and the pressure-input
// ghost columns (a uniform grid without them); the issue-bound FP32 path uses it whenever it can.
template <typename R, int NG, int FLUX, int RECON, bool EXT = true>
__device__ __forceinline__ void stage_tile(const StageArgs& A, const FluxConsts<R>& K, int bx,
                                           int by, unsigned char* smem_raw) {
  constexpr int RING = 2 * NG;
  const int T = blockDim.x, W = T - 2 * NG, t = threadIdx.x;
  const int x0 = bx * W;
  const int gx = x0 - NG + t;
  const int y0 = by * A.rows_per_cta;
  const int y1 = min(y0 + A.rows_per_cta, A.nj);
  R* ring = reinterpret_cast<R*>(smem_raw);  // [RING][4][T]
  R* sfi = ring + RING * 4 * T;              // [4][T]   i-edge between cols t and t+1
  R* sfj = sfi + 4 * T;                      // [2][4][T] j-edge between rows j and j+1 at slot j&1

  const R g = R(A.gamma), g1 = R(A.gamma - 1.0);
  bool flipx;
  const int sx = map_index(min(gx, A.ni + NG - 1), A.ni, A.bc[SIDE_MX], A.bc[SIDE_PX], flipx);
  // +x outlet / pressure-input ghost columns get the boundary state (lowest-priority BCs)
  const int xmode = gx < A.ni ? 0
                    : (A.bc[SIDE_PX] == BC_OUTLET
                           ? 1
                           : (EXT && A.bc[SIDE_PX] == BC_PRESSURE_INPUT ? 2 : 0));
  const bool in_i_edge = (t >= NG - 1) && (t <= NG + W - 1) && (gx <= A.ni - 1);
  const bool in_cell = (t >= NG) && (t <= NG + W - 1) && (gx < A.ni);
  const double dt = *A.dt;
  const double cc = A.coef * dt;
  [[maybe_unused]] const float ccf = (float)cc;  // mixed: the stage increment c L in FP32
  [[maybe_unused]] const float cfl_f = (float)A.cfl;
  const R* rp[6];
  // mixed_df constants of the update (unused by the other paths)
  [[maybe_unused]] df dx_inv, dy_inv, cfl_df, cc_df;
  if constexpr (Prec<R>::kind == 2) {
    dx_inv = to_df(A.G.rdxc ? A.G.rdxc[min(max(gx, 0), A.ni - 1)] : 1.0 / A.G.dx);
    dy_inv = to_df(1.0 / A.G.dy);
    cfl_df = to_df(A.cfl);
    cc_df = to_df(cc);
  }
  // FP32 reciprocal cell width of this thread's column (mixed path)
  [[maybe_unused]] const float idx_col =
      (EXT && A.G.rdxf) ? A.G.rdxf[min(max(gx, 0), A.ni - 1)] : (float)(1.0 / A.G.dx);
  // FP32 reciprocal row height of a uniform grid (one FP64 division per thread, not per row)
  [[maybe_unused]] const float idy_uni = (float)(1.0 / A.G.dy);

  // prologue: rows y0-NG .. y0+NG-1
  for (int r = y0 - NG; r < y0 + NG; ++r) {
    RowSrc<R> s;
    load_src<R>(A, sx, r, s);
    R q[4];
    src_to_prim<R>(A, s, flipx, xmode, r, g, g1, q);
    R* row = ring + slot_of<RING>(r) * 4 * T;
#pragma unroll
    for (int k = 0; k < 4; ++k) row[k * T + t] = q[k];
  }
  __syncthreads();
  if (in_cell && y0 < y1) {
    R F[4];
    ring_rows<R, RING>(ring, T, y0 - 1, rp);
    edge_flux<R, NG, FLUX, RECON, 1>(rp, T, A.limiter, t, K, F);
#pragma unroll
    for (int k = 0; k < 4; ++k) sfj[(((y0 - 1) & 1) * 4 + k) * T + t] = F[k];
  }
  __syncthreads();

  RowSrc<R> pre;
  if (y0 < y1) load_src<R>(A, sx, y0 + NG, pre);

  double dt_loc = INFINITY;
  int st_loc = 0;

  for (int j = y0; j < y1; ++j) {
    // operands of this row's cell update, issued early
    const size_t cidx = (size_t)j * A.pitch + (size_t)min(max(gx, 0), A.ni - 1);
    double ua[4], uk[4];
    if (in_cell) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        ua[k] = A.Ua[k] ? A.Ua[k][cidx] : 0.0;  // may alias Uo: plain load, read before write
        uk[k] = (A.kind == 1) ? __ldg(A.Uk[k] + cidx) : 0.0;
      }
    }
    RowSrc<R> nxt;
    if (j + 1 < y1) load_src<R>(A, sx, j + 1 + NG, nxt);
    {
      R q[4];
      src_to_prim<R>(A, pre, flipx, xmode, j + NG, g, g1, q);
      R* row = ring + slot_of<RING>(j + NG) * 4 * T;
#pragma unroll
      for (int k = 0; k < 4; ++k) row[k * T + t] = q[k];
    }
    pre = nxt;
    __syncthreads();
    ring_rows<R, RING>(ring, T, j, rp);
    if (in_i_edge) {
      R F[4];
      edge_flux<R, NG, FLUX, RECON, 0>(rp, T, A.limiter, t, K, F);
#pragma unroll
      for (int k = 0; k < 4; ++k) sfi[k * T + t] = F[k];
    }
    if (in_cell) {
      R F[4];
      edge_flux<R, NG, FLUX, RECON, 1>(rp, T, A.limiter, t, K, F);
#pragma unroll
      for (int k = 0; k < 4; ++k) sfj[((j & 1) * 4 + k) * T + t] = F[k];
    }
    __syncthreads();
    if (in_cell) {
      double un[4];
      // the cell's metrics (constants on a uniform grid)
      const Geom cg = cell_geom(A.G, gx, j);
      if constexpr (Prec<R>::kind == 2) {
        if (A.G.rdyc) dy_inv = to_df(A.G.rdyc[j]);
      }
      if constexpr (Prec<R>::kind != 1) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const R Fi = sfi[k * T + t], Fim = sfi[k * T + t - 1];
          const R Fj = sfj[((j & 1) * 4 + k) * T + t];
          const R Fjm = sfj[(((j - 1) & 1) * 4 + k) * T + t];
          double r;
          if constexpr (Prec<R>::kind == 0) {
            double L = divergence_fp64(Fi, Fim, Fj, Fjm, cg);
            if (k == 3 && A.src_q) L = L + A.src_q[cidx];
            if (A.kind == 2) {
              r = L;
            } else if (A.kind == 0) {
              r = ua[k] + __dmul_rn(L, cc);
              if (abs_lt(r, Num<double>::eps)) r = 0.0;
            } else {
              double s = __dmul_rn(ua[k], A.a) + __dmul_rn(uk[k], A.b);
              if (abs_lt(s, Num<double>::eps)) s = 0.0;
              r = s + __dmul_rn(L, cc);
              if (abs_lt(r, Num<double>::eps)) r = 0.0;
            }
          } else {
            // double-float divergence (pairs on the FP32 pipe) carried to FP64 once; the RK
            // accumulation in FP64: U^n + c L, or a U^n + b U^k + c L as two FP64 FMAs with the
            // increment c L formed in double-float: three FP64 operations per variable instead
            // of six (stages 2 and 3 of SSP-RK3 on the 4096^2 quadrant: 6 % faster)
            const df Ld = -((Fi - Fim) * dx_inv + (Fj - Fjm) * dy_inv);
            const bool src = k == 3 && A.src_q;
            if (A.kind == 2) {
              r = from_df(Ld);
              if (src) r = r + A.src_q[cidx];
            } else if (A.kind == 0) {
              double L = from_df(Ld);
              if (src) L = L + A.src_q[cidx];
              r = ua[k] + __dmul_rn(L, cc);
              if (abs_lt(r, Num<double>::eps)) r = 0.0;
            } else {
              const double d = src ? __dmul_rn(from_df(Ld) + A.src_q[cidx], cc)
                                   : from_df(Ld * cc_df);
              r = fma(uk[k], A.b, fma(ua[k], A.a, d));
              if (abs_lt(r, Num<double>::eps)) r = 0.0;
            }
          }
          un[k] = r;
          A.Uo[k][cidx] = r;
        }
      } else {
        // FP32 divergence and stage increment c L; the stage combine (the RK accumulation)
        // in FP64
        const float idx_f = idx_col;
        const float idy_f = (EXT && A.G.rdyf) ? A.G.rdyf[j] : idy_uni;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          float Fi = sfi[k * T + t], Fim = sfi[k * T + t - 1];
          float Fj = sfj[((j & 1) * 4 + k) * T + t];
          float Fjm = sfj[(((j - 1) & 1) * 4 + k) * T + t];
          float Lf = -((Fi - Fim) * idx_f + (Fj - Fjm) * idy_f);
          if (EXT && k == 3 && A.src_q) Lf = Lf + d2f_int(A.src_q[cidx]);
          double r;
          if (A.kind == 2) r = f2d_int(Lf);
          else if (A.kind == 0) r = ua[k] + f2d_int(Lf * ccf);
          else r = fma(uk[k], A.b, fma(ua[k], A.a, f2d_int(Lf * ccf)));
          un[k] = r;
          A.Uo[k][cidx] = r;
        }
      }
      if (A.last) {
        // CFL dt of the new state (get_timestep, mod_fluid.f90:554-558) and the sanity checks
        if constexpr (Prec<R>::kind == 0) {
          double u, v, p, cs;
          prim_from_cons(A.gamma, A.gamma - 1.0, un[0], un[1], un[2], un[3], u, v, p, cs);
          double d = div_rn(A.cfl, div_rn(fabs(u) + cs, cg.dx) + div_rn(fabs(v) + cs, cg.dy));
          if (d_less(d, dt_loc)) dt_loc = d;
          if (d_isnan(un[0]) || d_isnan(u) || d_isnan(v) || d_isnan(p)) st_loc |= ST_NAN;
          if (lt0(un[0])) st_loc |= ST_NEG_DENSITY;
          if (lt0(p)) st_loc |= ST_NEG_PRESSURE;
        } else if constexpr (Prec<R>::kind == 2) {
          df u, v, p, cs;
          const df rE = to_df(un[3]);
          prim_from_cons(g, g1, to_df(un[0]), to_df(un[1]), to_df(un[2]), rE, u, v, p, cs, true);
          if (near_vacuum(p.hi, rE.hi, 1e-4f)) {  // the FP64 recovery decides p and its sign
            double u64, v64, p64;
            prim_from_cons_f64(A.gamma, un[0], un[1], un[2], un[3], u64, v64, p64);
            u = to_df(u64); v = to_df(v64); p = to_df(p64);
            cs = df_sqrt(g * df_div(p, to_df(un[0])));
          }
          const df d = df_div(cfl_df, (df_abs(u) + cs) * dx_inv + (df_abs(v) + cs) * dy_inv);
          const double dd = from_df(d);
          if (dd > 0.0 && dd < dt_loc) dt_loc = dd;
          if (isnan(un[0]) || isnan(u.hi) || isnan(v.hi) || isnan(p.hi)) st_loc |= ST_NAN;
          if (un[0] < 0.0) st_loc |= ST_NEG_DENSITY;
          if (p.hi < 0.0f) st_loc |= ST_NEG_PRESSURE;
        } else {
          const float4 uf = make_float4(d2f_fast(un[0]), d2f_fast(un[1]), d2f_fast(un[2]),
                                        d2f_fast(un[3]));
          float u, v, p, cs;
          prim_from_cons(g, g1, uf.x, uf.y, uf.z, uf.w, u, v, p, cs);
          float d = cfl_f / ((fabsf(u) + cs) * idx_col +
                             (fabsf(v) + cs) * ((EXT && A.G.rdyf) ? A.G.rdyf[j] : idy_uni));
          double dd = f2d_int(d);
          if (__double_as_longlong(dd) < __double_as_longlong(dt_loc) && d > 0.0f) dt_loc = dd;
          // NaN and sign tests on the FP64 state itself (the fast conversion keeps neither)
          if (d_isnan(un[0]) || d_isnan(un[1]) || d_isnan(un[2]) || d_isnan(un[3]) ||
              isnan(u) || isnan(v) || isnan(p))
            st_loc |= ST_NAN;
          if (lt0(un[0])) st_loc |= ST_NEG_DENSITY;
          if (p < 0.0f) st_loc |= ST_NEG_PRESSURE;
        }
      }
    }
  }

  if (A.last) {
    // block min of dt (bits of positive doubles order as unsigned integers) and status OR
    unsigned long long bits =
        (dt_loc > 0.0) ? (unsigned long long)__double_as_longlong(dt_loc) : ~0ULL;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long ob = __shfl_xor_sync(0xffffffffu, bits, o);
      bits = ob < bits ? ob : bits;
      st_loc |= __shfl_xor_sync(0xffffffffu, st_loc, o);
    }
    if ((t & 31) == 0) {
      if (bits != ~0ULL) atomicMin(A.dt_min, bits);
      if (st_loc) atomicOr(A.status, st_loc);
    }
  }
}

// Minimum resident 256-thread CTAs per SM requested from the register allocator for the
// double-float kernels (their pair arithmetic is latency-bound; more warps hide it).
#ifndef CATO_DF_MIN_BLOCKS
#define CATO_DF_MIN_BLOCKS 2
#endif
// the same for the FP32 (mixed) kernels: the single-grid kernels run best unconstrained, the
// persistent batch kernels at 4 CTAs per SM (64 registers; +4.5 % on the batched workload)
#ifndef CATO_F32_MIN_BLOCKS
#define CATO_F32_MIN_BLOCKS 1
#endif
#ifndef CATO_F32_BATCH_MIN_BLOCKS
#define CATO_F32_BATCH_MIN_BLOCKS 4
#endif
// and for the FP64 kernels, which come in three register budgets (kernel variants 0, 1, 2): the
// compiler's choice, at most 128 registers (two 256-thread CTAs per SM) and at most 85 (three).
// Which is faster depends on the flux, the reconstruction, the plan and the flow
// (cato_gpu_tune measures it; the 4096^2 quadrant and Kelvin-Helmholtz grids run best with 85
// registers in 256-thread strips of 16 rows: +3 % and +4 % over the best 128-register plan);
// all give bit-identical results.
#ifndef CATO_F64_MIN_BLOCKS
#define CATO_F64_MIN_BLOCKS 1
#endif
#ifndef CATO_F64_MIN_BLOCKS_ALT
#define CATO_F64_MIN_BLOCKS_ALT 2
#endif
#ifndef CATO_F64_MIN_BLOCKS_ALT2
#define CATO_F64_MIN_BLOCKS_ALT2 3
#endif
template <typename R> constexpr int min_blocks() {
  return Prec<R>::kind == 2 ? CATO_DF_MIN_BLOCKS
                            : (Prec<R>::kind == 1 ? CATO_F32_MIN_BLOCKS : CATO_F64_MIN_BLOCKS);
}
// the persistent batch kernels (256-thread CTAs) run best with more resident warps than the
// single-grid kernels: FP64 and double-float at most 85 registers (3 CTAs per SM), measured on
// the batched random-circle workload (SLAU + MLP5) at +28 % (FP64, over the compiler's 229
// registers) and +21 % (double-float, over 122); both spill a little to the stack.  FP64 at 128
// registers gave +20 %, double-float at 64 less than at 85.
#ifndef CATO_F64_BATCH_MIN_BLOCKS
#define CATO_F64_BATCH_MIN_BLOCKS 3
#endif
#ifndef CATO_DF_BATCH_MIN_BLOCKS
#define CATO_DF_BATCH_MIN_BLOCKS 3
#endif
// FP64 M-AUSMPW+ (two interpolators' edge states live at once) spills too much at 85: at most
// 128 registers (205 against 168 M cell-updates/s); Roe and the other fluxes measured best at 85
#ifndef CATO_F64_BATCH_MIN_BLOCKS_MAUSMPW
#define CATO_F64_BATCH_MIN_BLOCKS_MAUSMPW 2
#endif
template <typename R, int FLUX> constexpr int batch_min_blocks() {
  return Prec<R>::kind == 2
             ? CATO_DF_BATCH_MIN_BLOCKS
             : (Prec<R>::kind == 1 ? CATO_F32_BATCH_MIN_BLOCKS
                                   : (FLUX == FLUX_M_AUSMPW ? CATO_F64_BATCH_MIN_BLOCKS_MAUSMPW
                                                            : CATO_F64_BATCH_MIN_BLOCKS));
}

template <typename R, int NG, int FLUX, int RECON, bool EXT, int MB>
__global__ void __launch_bounds__(256, MB)
    stage_kernel(const StageArgs A, const FluxConsts<R> K) {
  if (A.active && *A.active == 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  stage_tile<R, NG, FLUX, RECON, EXT>(A, K, blockIdx.x, blockIdx.y, smem_raw);
}

// whether a stage needs the EXT kernel (rectilinear grid, energy source, pressure input)
inline bool stage_needs_ext(const StageArgs& A) {
  return A.G.dxc != nullptr || A.src_q != nullptr || A.bc[SIDE_PX] == BC_PRESSURE_INPUT;
}

// dynamic shared memory of one CTA
template <typename R> inline size_t stage_smem_bytes(int T, int ng) {
  return sizeof(R) * (size_t)T * (2 * ng * 4 + 4 + 8);
}

}  // namespace cato
