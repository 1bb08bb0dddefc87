/*
 * cato_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference (smillerc/fvleg_2d, "CATO") FP64 time-step arithmetic,
 * used as the parity checker for the CUDA path and as the timed CPU baseline.  Nothing in
 * the product links against this library; only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it.
 *
 * Arrays are real64 Fortran column-major, halo-padded (1-ng:ni+ng, 1-ng:nj+ng), pointer to
 * element (1-ng,1-ng), leading dimension ni+2ng, exactly as field_2d_t%data.
 */
#ifndef CATO_ORACLE_H
#define CATO_ORACLE_H

#include <stdint.h>
#include "../include/cato_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_fluid oracle_fluid;

int oracle_set_threads(int n);
int oracle_config_default(cato_config* cfg, int32_t ni, int32_t nj);
int oracle_config_check(const cato_config* cfg);
int oracle_get_threads(void);

/* Pieces (each cites the reference routine it restates in cato_oracle.c). */
double oracle_limiter(int32_t limiter, double r);
void oracle_quad_metrics(const double x[4], const double y[4], double* volume,
                         double edge_lengths[4], double edge_norm_vectors[8],
                         double* min_dx, double* min_dy);
int oracle_apply_bc(const cato_config* cfg, double* rho, double* u, double* v, double* p);
int oracle_apply_bc_side(const cato_config* cfg, int side, int type, int do_corners, double* rho,
                         double* u, double* v, double* p);
int oracle_interpolate_edges(const cato_config* cfg, const double* q, double* i_edges,
                             double* j_edges);
int oracle_solve(const cato_config* cfg, double* rho, double* u, double* v, double* p,
                 double* d_rho_dt, double* d_rho_u_dt, double* d_rho_v_dt, double* d_rho_E_dt);
/* oracle_solve on the rectilinear grid of node coordinates x(1..ni+1), y(1..nj+1). */
int oracle_solve_rect(const cato_config* cfg, const double* x_nodes, const double* y_nodes,
                      double* rho, double* u, double* v, double* p, double* d_rho_dt,
                      double* d_rho_u_dt, double* d_rho_v_dt, double* d_rho_E_dt);

/* Whole fluid_t. */
oracle_fluid* oracle_create(const cato_config* cfg);
void oracle_destroy(oracle_fluid* f);
/* allow_subcycle and subcycle_tolerance of the deck's [time] section */
int oracle_set_subcycle(oracle_fluid* f, int allow, double tolerance);
/* Slab of a row-split grid (CATO_BC_EXCHANGE sides): fn(user, rho, u, v, p) receives the
 * halo-padded primitives of every residual evaluation before its boundary conditions and fills
 * the ghost rows beyond the exchange sides (interior columns) with the neighbours' rows. */
typedef void (*oracle_exchange_fn)(void* user, double* rho, double* u, double* v, double* p);
int oracle_set_exchange(oracle_fluid* f, oracle_exchange_fn fn, void* user);
/* dt of the last step (after any subcycling) */
double oracle_dt(const oracle_fluid* f);
int oracle_set_primitive(oracle_fluid* f, const double* rho, const double* u, const double* v,
                         const double* p);
double oracle_get_timestep(oracle_fluid* f);
int oracle_integrate(oracle_fluid* f, double dt, int32_t* error_code);
int oracle_get_state(oracle_fluid* f, double* rho, double* rho_u, double* rho_v, double* rho_E,
                     double* u, double* v, double* p, double* cs);
int oracle_set_conserved(oracle_fluid* f, const double* rho, const double* rho_u,
                         const double* rho_v, const double* rho_E);
double oracle_time(oracle_fluid* f);
int64_t oracle_iteration(oracle_fluid* f);
/* calculate_convergence of the last step (CATO_ERR_STATE before the first step) */
int oracle_convergence(oracle_fluid* f, double out[4]);
/* interior totals of rho, rho u, rho v, rho E times the cell volume */
int oracle_conservation_sums(oracle_fluid* f, double out[4]);
int oracle_set_rectilinear(oracle_fluid* f, const double* x_nodes, const double* y_nodes);
int oracle_set_time(oracle_fluid* f, double time, int64_t iteration);
/* powers of the pressure-input inlet: 0 = libm pow (as the reference), 1 = correctly rounded */
int oracle_set_pow_mode(int mode);
int oracle_set_energy_source(oracle_fluid* f, const cato_energy_source* src, int32_t n,
                             const double* t, const double* v, const double* crit);
int oracle_source_field(oracle_fluid* f, double* out);
double oracle_pow(int mode, double x, double y);
int oracle_set_bc_table(oracle_fluid* f, int32_t n, const double* t, const double* p,
                        const double* rho);
/* oracle_solve with a pressure-input table evaluated at `time` */
int oracle_solve_pbc(const cato_config* cfg, int32_t n, const double* t, const double* pt,
                     const double* rhot, double time, double* rho, double* u, double* v,
                     double* p, double* d_rho_dt, double* d_rho_u_dt, double* d_rho_v_dt,
                     double* d_rho_E_dt);

#ifdef __cplusplus
}
#endif
#endif
