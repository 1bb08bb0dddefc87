// cato_setup.cuh -- host-side derivations shared by every entry point that turns a cato_config
// into kernel arguments (handles, batch slots and the allocation-free residual), so that all of
// them feed the stage kernel the same constants and launch shape for the same configuration.
#pragma once

#include "../../include/cato_gpu.h"
#include "cato_physics.cuh"

namespace cato {

// The scheme constants of a configuration (gamma-derived ratios, AUSM+-up coefficients, the
// low-Mach and entropy-fix switches), in FP64; other compute types take convert_consts of it.
inline FluxConsts<double> flux_consts_of(const cato_config& c) {
  const double g = c.gamma;
  FluxConsts<double> K{};
  K.gamma = g;
  K.g_over_gm1 = g / (g - 1.0);
  K.gm1 = g - 1.0;
  K.two_gm1_over_gp1 = 2.0 * ((g - 1.0) / (g + 1.0));
  K.gamma_factor = ((2.0 * (g - 1.0)) / (g + 1.0));
  K.hllc_gf = (g + 1.0) / (2.0 * g);
  K.harten_delta = c.harten_delta;
  K.ausm_beta = c.ausm_beta;
  K.ausm_kp = c.ausm_kp;
  K.ausm_ku = c.ausm_ku;
  K.ausm_sigma = c.ausm_sigma;
  K.low_mach_fix = c.apply_low_mach_fix ? 1 : 0;
  K.harten = c.roe_entropy_fix == CATO_ROE_HARTEN ? 1 : 0;
  return K;
}

// Default single-grid launch shape: wide strips for large grids; narrow strips and short marches
// for small grids so that the launch fills the 152 SMs; narrow strips when a wide one would be
// wider than the grid with its halo.
struct LaunchShape {
  int threads;
  int rows_per_cta;
};
inline LaunchShape default_shape(int ni, int nj, int ng) {
  const long long cells = (long long)ni * nj;
  LaunchShape p;
  if (cells < 200000) { p.threads = 64; p.rows_per_cta = 8; }
  else if (cells < 4000000) { p.threads = 128; p.rows_per_cta = 32; }
  else { p.threads = 128; p.rows_per_cta = 64; }
  if (p.threads - 2 * ng > ni + 2 * ng) p.threads = 64;
  return p;
}

// reconstruction kind of a limiter id: 0 = TVD2, 3 = MLP3, 5 = MLP5
inline int recon_of_limiter(int limiter) {
  return limiter == CATO_LIM_MLP3 ? 3 : (limiter == CATO_LIM_MLP5 ? 5 : 0);
}

}  // namespace cato
