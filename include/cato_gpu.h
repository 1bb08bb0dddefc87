/*
 * cato_gpu.h -- C-ABI of the GB300 (sm_103a) implementation of CATO's time-step hot path.
 *
 * One handle is one 2-D structured grid instance whose state lives in device memory (HBM)
 * between calls.  Host arrays crossing this boundary use the reference's field_2d_t layout:
 * real64, Fortran column-major (i fastest), halo-padded with bounds
 * (1-n_ghost : ni+n_ghost, 1-n_ghost : nj+n_ghost)   [src/lib/field/field_2d.f90:58-64].
 * A pointer argument points at element (1-n_ghost, 1-n_ghost); `ld` is the leading dimension
 * (>= ni + 2*n_ghost).  Only interior cells are read on upload.
 *
 * Every entry point returns CATO_OK (0) or a negative-free error code and never aborts; the
 * reference instead stops the program (`error stop`, src/lib/error.f90:33-35).  A handle is
 * used by one host thread at a time; different handles are independent (no global state: the
 * reference's singleton EOS, src/lib/equation_of_state.f90:70, becomes per-handle gamma).
 */
#ifndef CATO_GPU_H
#define CATO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Return / error codes.  1..3 are the reference's fluid error codes (src/lib/error.f90:6-9). */
enum cato_status {
  CATO_OK = 0,
  CATO_NEG_DENSITY = 1,
  CATO_NEG_PRESSURE = 2,
  CATO_NANS_FOUND = 3,
  CATO_ERR_CONFIG = 10,   /* invalid configuration (unknown flux/limiter, bad ghost count, ...) */
  CATO_ERR_OOM = 11,      /* device allocation failed */
  CATO_ERR_CUDA = 12,     /* CUDA runtime error (message via cato_gpu_last_error) */
  CATO_ERR_ARG = 13,      /* bad argument (null pointer, too-small leading dimension, ...) */
  CATO_ERR_TIMEOUT = 14,  /* a bounded device-side wait gave up */
  CATO_ERR_STATE = 15,    /* call out of order (e.g. integrate before upload) */
  CATO_ERR_CAPACITY = 16, /* the request exceeds a fixed-size device buffer (no-alloc entry) */
  CATO_ERR_BC_INPUT = 17  /* the pressure-input target pressure or density is below tiny at a
                             stage's time (the reference stops, pressure_input_bc.f90:225-253) */
};

/* Flux solvers.  Names as accepted by the reference deck key [scheme] flux_solver
 * (src/lib/fluid/mod_fluid.f90:223-238); AUSM+-up and HLLC have no runnable reference. */
enum cato_flux {
  CATO_FLUX_AUSMPW_PLUS = 0,  /* 'AUSMPW+'   ausmpw_plus_solver.fypp:214-463 */
  CATO_FLUX_SLAU = 1,         /* 'SLAU'      slau_solver.fypp:253-494 */
  CATO_FLUX_SLAU2 = 2,        /* 'SLAU2' */
  CATO_FLUX_SD_SLAU = 3,      /* 'SD-SLAU' */
  CATO_FLUX_SD_SLAU2 = 4,     /* 'SD-SLAU2' */
  CATO_FLUX_ROE = 5,          /* 'Roe'       roe_solver.fypp:229-515 */
  CATO_FLUX_AUSM_PLUS_UP = 6, /* 'AUSM+-up'  ausm_plus_solver.f90:394-643 (driver restated) */
  CATO_FLUX_HLLC = 7,         /* 'HLLC'      Toro HLLC, PVRS wave speeds (reference is a stub) */
  CATO_FLUX_M_AUSMPW_PLUS = 8 /* 'M-AUSMPW+' m_ausmpw_plus_solver.fypp:437-708 (superbee-blended
                                 interface states) */
};

/* Edge reconstruction (src/lib/spatial_reconstruction/muscl_factory.f90:54-94). */
enum cato_limiter {
  CATO_LIM_MINMOD = 0,   /* muscl_tvd2.fypp:195-197 */
  CATO_LIM_SUPERBEE = 1, /* muscl_tvd2.fypp:197-199 */
  CATO_LIM_VAN_LEER = 2, /* muscl_tvd2.fypp:199-200 */
  CATO_LIM_MLP3 = 3,     /* muscl_mlp.fypp, ORDER=3 */
  CATO_LIM_MLP5 = 4      /* muscl_mlp.fypp, ORDER=5, needs n_ghost = 3 */
};

/* Time integration ([time] integration_strategy, mod_fluid.f90:424-446). */
enum cato_rk {
  CATO_RK_SSP2 = 0,  /* 'ssp_rk2'             mod_fluid.f90:1081-1160 */
  CATO_RK_SSP3 = 1,  /* 'ssp_rk3'|'ssp_rk33'  mod_fluid.f90:739-854 */
  CATO_RK_1_3 = 2,   /* 'rk(1,3)'  low-storage family, mod_fluid.f90:889-1007 */
  CATO_RK_1_4 = 3,
  CATO_RK_1_5 = 4,
  CATO_RK_2_3 = 5,
  CATO_RK_2_4 = 6,
  CATO_RK_2_5 = 7
};

/* Boundary conditions (src/lib/boundary_conditions/bc_factory.f90:39-66). */
enum cato_bc {
  CATO_BC_ZERO_GRADIENT = 0, /* priority 1, zero_gradient_bc.f90:54-121 */
  CATO_BC_SYMMETRY = 1,      /* priority 1, symmetry_bc.f90:56-133 */
  CATO_BC_PERIODIC = 2,      /* priority 2, periodic_bc.fypp:78-283 */
  CATO_BC_OUTLET = 3,        /* priority 0, outlet_bc.f90:63-176: characteristic subsonic outflow
                                to bc_pressure on +x, line copies on the other sides */
  CATO_BC_PRESSURE_INPUT = 4, /* priority 0, +x only, pressure_input_bc.f90:256-414: the
                                characteristic inlet/outlet state toward a target pressure and
                                density, constant (bc_pressure, bc_density) or tabulated in time
                                (cato_gpu_set_bc_table) */
  CATO_BC_EXCHANGE = 5       /* +-y only: not a boundary but the cut between two slabs of one
                                grid split by rows (one handle per GPU); the n_ghost rows beyond
                                it are the neighbouring slab's interior rows, copied in before
                                every stage (cato_gpu_halo_import), as the reference's coarray
                                images exchange their edges (field_2d.f90:551-654).  The x
                                boundaries treat these rows as interior rows. */
};

/* Sides in the reference's application order within one priority (flux_solver.f90:165-183). */
enum cato_side { CATO_PLUS_X = 0, CATO_PLUS_Y = 1, CATO_MINUS_X = 2, CATO_MINUS_Y = 3 };

enum cato_precision {
  CATO_FP64 = 0,   /* the drop-in path: IEEE FP64 throughout, reference operation order */
  CATO_MIXED = 1,  /* FP32 reconstruction + flux arithmetic, FP64 conserved state and RK update */
  CATO_MIXED_DF = 2 /* double-float (pairs of FP32, ~44-bit) reconstruction, flux and divergence
                       on the FP32 pipe; FP64 conserved and stage states and RK combine */
};

enum cato_roe_fix {
  CATO_ROE_REFERENCE = 0, /* as built: no entropy fix (roe_solver.fypp:460-465 commented) */
  CATO_ROE_HARTEN = 1     /* Harten fix of roe_solver.fypp:529-536 with delta = harten_delta * c~ */
};

typedef struct cato_config {
  int32_t ni, nj;             /* interior cells in i (x) and j (y) */
  int32_t n_ghost;            /* ghost layers: 2, or 3 for MLP5 (mod_input.f90:320-338) */
  int32_t flux;               /* enum cato_flux */
  int32_t limiter;            /* enum cato_limiter */
  int32_t rk;                 /* enum cato_rk */
  int32_t bc[4];              /* enum cato_bc, indexed by enum cato_side */
  int32_t apply_low_mach_fix; /* AUSMPW+ low-Mach fix; reference default true (mod_input.f90:134) */
  int32_t precision;          /* enum cato_precision */
  int32_t roe_entropy_fix;    /* enum cato_roe_fix */
  int32_t reserved0;
  double gamma;               /* [physics] polytropic_index */
  double cfl;                 /* [time] cfl */
  double dx, dy;              /* uniform Cartesian cell size (geometry of quad_cell.f90:69-229) */
  double harten_delta;        /* Harten delta coefficient (CATO_ROE_HARTEN only) */
  double ausm_beta;           /* [ausm] beta, default 1/8 */
  double ausm_kp;             /* [ausm] pressure_diffusion_coeff, default 0.25 */
  double ausm_ku;             /* K_u, default 0.75 (not read from the deck by the reference) */
  double ausm_sigma;          /* [ausm] sonic_point_sigma, default 1 */
  double bc_pressure;         /* [boundary_conditions] outflow_ambient_pressure (CATO_BC_OUTLET) or
                                 constant_bc_pressure_value x press_to_nondim (constant
                                 CATO_BC_PRESSURE_INPUT); the reference keeps both in one value */
  double bc_density;          /* [boundary_conditions] bc_density x density_to_dim: the constant
                                 CATO_BC_PRESSURE_INPUT target density */
} cato_config;

typedef struct cato_handle cato_handle;

/* Library version string. */
const char* cato_gpu_version(void);

/* Fill `cfg` with the reference's deck defaults (mod_input.f90:34-148) for an ni x nj grid. */
int cato_config_default(cato_config* cfg, int32_t ni, int32_t nj);

/* Validate a configuration without touching the GPU; returns CATO_OK or CATO_ERR_CONFIG. */
int cato_config_check(const cato_config* cfg);

/* Create / destroy a grid instance.  Replaces fluid_t%initialize + flux_solver_t%initialize
 * (mod_fluid.f90:159-254, flux_solver.f90:89-95).  Allocates the device state. */
int cato_gpu_create(const cato_config* cfg, cato_handle** out);
int cato_gpu_destroy(cato_handle* h);

/* Last error message of this handle (empty string if none). */
const char* cato_gpu_last_error(const cato_handle* h);

/* Upload primitive initial conditions (rho, u, v, p; interior of halo-padded arrays).
 * Replaces fluid_t%initialize_from_hdf5 + eos%primitive_to_conserved (mod_fluid.f90:339-363):
 * the conserved state is derived on the device; the first stage uses these primitives as is. */
int cato_gpu_upload_primitive(cato_handle* h, const double* rho, const double* u,
                              const double* v, const double* p, int64_t ld);

/* Rectilinear (tensor-product) grid: the interior node coordinates x(1..ni+1) and y(1..nj+1),
 * strictly increasing, in place of the configuration's uniform dx x dy.  Covers the uniform and
 * the layered grids of pycato (generate_initial_grids.py:43-113, 166-380), whose cells are
 * axis-aligned; the cell metrics follow quad_cell.f90:69-229 (volume, edge lengths with their
 * 2-eps snap, min_dx / min_dy per cell).  Replaces the grid part of
 * grid_block_2d_t%initialize (grid_block_2d.f90:54-151) for such grids.  Both pointers NULL
 * returns to the uniform grid.  The state must be uploaded (again) afterwards. */
int cato_gpu_set_rectilinear(cato_handle* h, const double* x_nodes, const double* y_nodes);

/* Energy source term ([source_terms], source_t of src/lib/source_terms/mod_source.f90:63-425):
 * q_dot_h added to the energy equation's right-hand side at every stage (time_derivative,
 * mod_fluid.f90:503), recomputed once per step from the step-start time and density
 * (source_t%integrate, :296-312). */
enum cato_source_geometry {
  CATO_SRC_UNIFORM = 0,     /* 'uniform' */
  CATO_SRC_CONSTANT_XY = 1, /* 'constant_xy' (the reference tests centroid_x > ylo) */
  CATO_SRC_GAUSSIAN_1D = 2, /* '1d_gaussian', constant in y, centred on the deposition column */
  CATO_SRC_DECAY = 3        /* 'decay' */
};

typedef struct cato_energy_source {
  int32_t geometry;        /* enum cato_source_geometry */
  int32_t gaussian_order;  /* source_gaussian_order (1d_gaussian) */
  double constant_value;   /* constant_source_value (apply_constant_source; used unscaled) */
  double multiplier;       /* source_scale_factor */
  double xlo, xhi, ylo, yhi;  /* constant_xy box, x len_to_nondim */
  double fwhm_x, fwhm_y;      /* 1d_gaussian widths, x len_to_nondim */
} cato_energy_source;

/* Turn the energy source on (src != NULL) or off.  n = 0: the constant value; n >= 2: the
 * table of read_input_file (mod_source.f90:127-258), already scaled: time x t_to_nondim,
 * value x pow_to_nondim, critical density x density_to_nondim (strictly increasing times).
 * Cell centroids come from the rectilinear nodes (cato_gpu_set_rectilinear), else from a
 * uniform grid with its first node at 0. */
int cato_gpu_set_energy_source(cato_handle* h, const cato_energy_source* src, int32_t n,
                               const double* time, const double* value,
                               const double* critical_density);

/* Target of a CATO_BC_PRESSURE_INPUT side as a table in time: n >= 2 points (time strictly
 * increasing), pressure and density already scaled as read_pressure_input does
 * (pressure_input_bc.f90:92-181: time x t_to_nondim, pressure x press_to_nondim x
 * bc_pressure_scale_factor, density x density_to_nondim x bc_pressure_scale_factor).  Evaluated
 * per stage as linear_interp_1d (finterp) at the stage's flux-solver time: t_n + dt, or for the
 * first stage of an rk(m,n) step the creation time (upload: 0, or cato_gpu_set_time) + dt; a
 * single cato_gpu_solve evaluates it at the handle's time.  n = 0 returns to the constant
 * target of the configuration. */
int cato_gpu_set_bc_table(cato_handle* h, int32_t n, const double* time, const double* pressure,
                          const double* density);

/* CFL time step of the current state.  Replaces fluid_t%get_timestep (mod_fluid.f90:518-562). */
int cato_gpu_get_timestep(cato_handle* h, double* dt);

/* Advance one time step.  Replaces fluid_t%integrate (mod_fluid.f90:411-450) as called by
 * master_puppeteer_t%integrate (master_puppeteer.f90:155-200): with dt <= 0 the CFL dt of the
 * current state is used (computed on the device), otherwise the given dt.  On return *dt_used
 * (may be NULL) holds the dt taken and *error_code (may be NULL) the fluid error code. */
int cato_gpu_integrate(cato_handle* h, double dt, double* dt_used, int32_t* error_code);

/* Run the time loop of src/main.f90:138-198 on the device without per-step host round trips:
 * CFL dt every step, stop once time >= t_end or after max_steps steps (no last-step trim).
 * Steps run in CUDA-graph chunks; the stop test is evaluated on the device. */
int cato_gpu_run(cato_handle* h, int64_t max_steps, double t_end, int64_t* steps_done,
                 double* time, int32_t* error_code);

/* Time bookkeeping (fluid_t%set_time, mod_fluid.f90:400-409).  set_time also sets the creation
 * time of the state, as a fluid_t created at that time (restart: new_fluid(..., time),
 * master_puppeteer.f90:132). */
int cato_gpu_set_time(cato_handle* h, double time, int64_t iteration);
int cato_gpu_get_time(cato_handle* h, double* time, int64_t* iteration, double* last_dt);

/* Download state into halo-padded host arrays (interior written, ghosts set to 0).  Any pointer
 * may be NULL.  u, v, p, cs are fluid_t's derived quantities (mod_fluid.f90:564-591). */
int cato_gpu_download(cato_handle* h, double* rho, double* rho_u, double* rho_v, double* rho_E,
                      double* u, double* v, double* p, double* cs, int64_t ld);

/* Global totals of the current state in FP64: sum over the interior of rho, rho u, rho v, rho E
 * times the cell volume (mass, momentum and energy in the domain; the reference sums rho_E for
 * its energy check, mod_fluid.f90:808-811).  Deterministic: a fixed partition and summation
 * tree, so repeated calls on the same state give the same bits. */
int cato_gpu_conservation_sums(cato_handle* h, double totals[4]);

/* calculate_convergence (mod_fluid.f90:1162-1205) of the last step: L2 norm of the change from
 * the first to the last stage over the interior, divided by the first stage's norm (by
 * max(norm, 1) for rho u and rho v): SSP-RK2 U_1 vs U_2, SSP-RK3 U_1 vs U_3, rk(m,n) U_0 vs
 * U_curr.  Computed on demand from the stage buffers of the last step (no cost per step).
 * CATO_ERR_STATE before the first step after an upload, and for rk(m,n) outside the mixed
 * path (the last stage overwrites U_0 in place there). */
int cato_gpu_convergence(cato_handle* h, double l2[4]);

/* flux_solver_t%solve (flux_solver.f90:66-87) on caller-given primitive fields: applies the BCs
 * to the ghosts of rho/u/v/p (written back, as the reference's intent(inout)), reconstructs,
 * computes edge fluxes and the flux divergence into d_*_dt (halo-padded, ghosts zeroed as in
 * flux_solver.f90:433-457).  Uses the handle's scheme; does not change the handle's state. */
int cato_gpu_solve(cato_handle* h, double* rho, double* u, double* v, double* p,
                   double* d_rho_dt, double* d_rho_u_dt, double* d_rho_v_dt, double* d_rho_E_dt,
                   int64_t ld);

/* muscl_interpolation_t%interpolate_edge_values (muscl_interpolation.f90:37-43) for one field
 * q whose ghosts are already filled.  Output layouts are the reference's:
 * i_edges(1:2, -1:ni, 0:nj) and j_edges(1:2, 0:ni, -1:nj), Fortran order, (1)=L (2)=R. */
int cato_gpu_interpolate_edges(cato_handle* h, const double* q, int64_t ld,
                               double* i_edges, double* j_edges);

/* Current device status word (bit 0: negative density, bit 1: negative pressure, bit 2: NaN). */
int cato_gpu_status(cato_handle* h, int32_t* status_bits);

/* Synchronise the handle's stream. */
int cato_gpu_synchronize(cato_handle* h);

/* Run all of this handle's work on `stream` (a cudaStream_t; NULL restores the handle's own
 * stream).  Lets a caller order the solver with its own work or time it with its own events. */
int cato_gpu_set_stream(cato_handle* h, void* stream);

/* One time step (CFL dt) with a CUDA event between kernels: kernel_ms[k] receives the device
 * time of kernel k (k = 0: step control, then one entry per RK stage).  The per-stage analogue
 * of the reference's timing.csv (src/lib/mod_timing.f90:35-128). */
int cato_gpu_profile_step(cato_handle* h, float* kernel_ms, int32_t capacity, int32_t* n_kernels);

/* Kernel launches per time step of this handle (step control + RK stages). */
int cato_gpu_launches_per_step(const cato_handle* h, int32_t* n);

/* Exactly n_steps CFL steps with no host round trip, timed with CUDA events on the handle's
 * stream: *total_ms = device time of all of them; kernel_ms (may be NULL, `capacity` entries)
 * accumulates per kernel slot (0: step control, k: RK stage k) over the steps. */
int cato_gpu_run_timed(cato_handle* h, int64_t n_steps, float* total_ms, float* kernel_ms,
                       int32_t capacity);

/* Work decomposition of the stage kernel (the autotuner's knobs): CTA width `threads` (a
 * multiple of 32 in [64, 256], including 2*n_ghost halo columns) and rows marched per CTA. */
int cato_gpu_set_plan(cato_handle* h, int32_t threads, int32_t rows_per_cta);
int cato_gpu_get_plan(const cato_handle* h, int32_t* threads, int32_t* rows_per_cta);

/* Register budget of the FP64 stage kernel (the third knob): 0 = the compiler's choice (fewer
 * resident warps, more registers each), 1 = at most 128 registers per thread, 2 = at most 85.
 * Which is faster depends on the flux, the reconstruction, the plan and the flow; the results
 * are bit-identical.  Accepted and ignored by the mixed precisions. */
int cato_gpu_set_kernel_variant(cato_handle* h, int32_t variant);
int cato_gpu_get_kernel_variant(const cato_handle* h, int32_t* variant);

/* Autotune the stage kernel on the live state: a few candidate plans (the current strip width
 * and 256-wide strips, each with the current, half and a quarter of the rows per CTA), each
 * with every FP64 register budget, run `steps` CFL steps each (timed with CUDA events), and the
 * fastest stays set.  These are real steps of the run
 * (the solution advances by *steps_taken steps, bit-identical whichever candidate runs them);
 * *best_ms = the fastest candidate's time per step.  Returns the first fluid error, if any. */
int cato_gpu_tune(cato_handle* h, int32_t steps, int32_t* steps_taken, float* best_ms);

/* Step options of the deck's [time] section.
 * keep_step_start: each step first copies U^n aside (one extra state, 32 B per cell, and a
 *   copy per step), so that cato_gpu_convergence also covers rk(m,n) steps, whose norms compare
 *   the last stage with U_0 = U^n (mod_fluid.f90:970); the residual history needs them.
 * allow_subcycle, subcycle_tolerance: subcycle_check (mod_fluid.f90:856-887): an SSP-RK2/3 step
 *   whose L2 convergence norms (calculate_convergence) exceed the tolerance in any variable is
 *   taken again from U^n with dt / 10, until they do not; the step's dt and the clock use the
 *   last dt.  rk(m,n) steps are not subcycled, as in the reference.  Implies keep_step_start.
 *   Not combined with the pressure-input boundary (CATO_ERR_CONFIG).
 * Off by default; with either on, cato_gpu_run takes its steps from the host. */
int cato_gpu_set_step_options(cato_handle* h, int32_t keep_step_start, int32_t allow_subcycle,
                              double subcycle_tolerance);

/* One time step taken stage by stage, for grids split into slabs by rows (CATO_BC_EXCHANGE
 * sides), whose ghost rows must be refreshed from the neighbouring slabs before every stage:
 *   cato_gpu_step_begin(h, dt);               dt > 0: this step's dt, e.g. the minimum of the
 *                                             slabs' cato_gpu_get_timestep (min_to_all,
 *                                             mod_collectives.f90:159-163); dt <= 0: own CFL dt
 *   repeat: halo export / exchange / import;  (the rows of the next stage's input)
 *           cato_gpu_step_stage(h, &left);    runs the next RK stage; left = stages still to run
 *   cato_gpu_step_end(h, &dt_used, &error_code);
 * The sequence of kernels is the one cato_gpu_integrate enqueues; any handle may use it.  Step
 * options (subcycling, the kept step start) are not combined with it.  On a slab,
 * cato_gpu_conservation_sums covers the slab's rows (the grid's totals are the sums over the
 * slabs) and cato_gpu_convergence gives the slab's own relative norms. */
int cato_gpu_step_begin(cato_handle* h, double dt);
int cato_gpu_step_stage(cato_handle* h, int32_t* stages_left);
int cato_gpu_step_end(cato_handle* h, double* dt_used, int32_t* error_code);

/* Edge rows of the next stage's input for the slab exchange.  side: CATO_PLUS_Y or
 * CATO_MINUS_Y, which must be a CATO_BC_EXCHANGE side.  rows: 4 fields (rho, rho u, rho v, rho E;
 * or the primitives rho, u, v, p before the first stage after an upload) x n_ghost rows (in
 * increasing j) x ni columns, contiguous doubles.  export copies out the n_ghost interior rows
 * next to `side`; import writes the n_ghost ghost rows beyond `side` (the neighbour's export of
 * its opposite side).  Between cato_gpu_step_begin and the last cato_gpu_step_stage, or before
 * a step (then the rows of the first stage's input). */
int cato_gpu_halo_export(cato_handle* h, int32_t side, double* rows);
int cato_gpu_halo_import(cato_handle* h, int32_t side, const double* rows);

/* Select the CUDA device used by handles created afterwards on this host thread. */
int cato_gpu_select_device(int32_t device);

/* Device self-check of the FP64 path's IEEE division and square root, which run on the integer
 * pipe (GB300's FP64 pipe is 1/64 of the FP32 rate): n seeded operand pairs (random bit patterns,
 * narrow exponent ranges, divisors with few significand bits, quotients near 1) go through the
 * integer routines and the hardware instructions on the current device.  tested[0] / tested[1]:
 * the divisions / square roots the integer routines took (the rest fall back to the hardware),
 * mismatches[0] / mismatches[1]: how many of those differ in any bit.  seed_ulps[0] / [1]: the
 * largest distance, in FP32 units in the last place and over every input, of the hardware
 * reciprocal / reciprocal-square-root approximations that seed the routines from the correctly
 * rounded values (the routines are verified on the host for seeds up to 8 ulps off).  No
 * counterpart in the reference. */
int cato_gpu_check_divsqrt(int64_t n, uint64_t seed, uint64_t tested[2], uint64_t mismatches[2],
                           int32_t seed_ulps[2]);

/* cato_gpu_solve for callers that cannot allocate device memory: no handle, no cudaMalloc or
 * cudaFree.  It has no counterpart in the reference; it serves callers whose device memory is
 * owned by another allocator (a framework pool, a fixed HBM budget) and callers in
 * latency-critical loops where an allocation could synchronize the device.  Same arguments and
 * results as cato_gpu_solve (host arrays, BC ghosts written back), FP64 schemes only.  All device
 * memory is one fixed 32 MiB array per GPU: grids needing more than
 * 8*pitch*nj + 4*(ni+2ng)*(nj+2ng) + 32 doubles (pitch = ni rounded up to 32; 512 x 512 fits)
 * are refused with CATO_ERR_CAPACITY.  The first call on a device sets up the array's address
 * (cudaGetSymbolAddress) and should come before any stream capture; that address belongs to the
 * device's primary context, so the entry point must not be called on a device after
 * cudaDeviceReset of it.  Calls share the array and would race if they overlapped on the GPU, so
 * each call locks its device, runs on the calling thread's per-thread default stream
 * (cudaStreamPerThread: it neither waits for nor blocks the process's other streams) and
 * synchronizes it before returning. */
int cato_gpu_solve_noalloc(const cato_config* cfg, double* rho, double* u, double* v, double* p,
                           double* d_rho_dt, double* d_rho_u_dt, double* d_rho_v_dt,
                           double* d_rho_E_dt, int64_t ld);

/* ---- Batched engine: many independent instances of uneven sizes advanced together ---------
 * No counterpart in the reference (CATO runs one grid per process).  Each instance keeps its
 * own CFL dt, time, iteration count and stop condition; one step of the batch is one persistent
 * launch per RK stage and per (flux, reconstruction) group, whose CTAs pull (instance, tile)
 * work items from a device queue.  Chunks of steps are captured in a CUDA graph.  An instance's
 * results do not depend on the other instances in the batch. */
typedef struct cato_batch cato_batch;

/* A batch of at most `capacity` instances, all with `precision` and integrator `rk`. */
int cato_batch_create(int32_t capacity, int32_t precision, int32_t rk, cato_batch** out);
int cato_batch_destroy(cato_batch* b);

/* Device bytes one instance of `cfg` occupies (state, stage buffers), for admission control. */
int cato_batch_instance_bytes(const cato_config* cfg, uint64_t* bytes);

/* Add an instance from primitive initial conditions (as cato_gpu_upload_primitive); it runs
 * until time >= t_end or max_steps steps (max_steps < 0: no limit).  *slot identifies it. */
int cato_batch_add(cato_batch* b, const cato_config* cfg, const double* rho, const double* u,
                   const double* v, const double* p, int64_t ld, double t_end, int64_t max_steps,
                   int32_t* slot);
int cato_batch_remove(cato_batch* b, int32_t slot);

/* Tile plan shared by all instances (CTA width incl. halo, rows per tile). */
int cato_batch_set_plan(cato_batch* b, int32_t threads, int32_t rows_per_cta);

/* Advance every running instance n_steps steps (instances that reach their stop condition idle);
 * with use_graph, whole chunks replay a captured CUDA graph.  *device_ms = event time. */
int cato_batch_step(cato_batch* b, int32_t n_steps, int32_t use_graph, float* device_ms);

/* One instance's progress; *running = 0 once it reached t_end / max_steps or failed. */
int cato_batch_query(cato_batch* b, int32_t slot, int64_t* iteration, double* time, double* dt,
                     int32_t* running, int32_t* error_code);

/* Number of running instances; running_flags (capacity entries, may be NULL) per slot. */
int cato_batch_running(cato_batch* b, int32_t* n_running, int32_t* running_flags);

/* Conserved state of one instance into halo-padded host arrays (any may be NULL). */
int cato_batch_download(cato_batch* b, int32_t slot, double* rho, double* rho_u, double* rho_v,
                        double* rho_E, int64_t ld);

/* Page-locked host memory for fast uploads/downloads (cudaHostAlloc / cudaFreeHost). */
int cato_host_alloc(uint64_t bytes, void** out);
int cato_host_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* CATO_GPU_H */
