// cato_capi.cu -- the C-ABI of include/cato_gpu.h: handles, device state, step sequencing.
//
// Device layout of one instance (all interior-only, row-major with i fastest = the reference's
// Fortran (i, j) order, row pitch rounded up to 32 elements so every row starts 256-B aligned),
// the same for every precision: U^n (4 x f64) + two stage buffers S0, S1 (4 x f64 each).  The
// last stage writes U^{n+1} over U^n in place (U^n is only read point-wise there).  The stage
// combine (the RK accumulation) is FP64 in every precision; reconstruction, flux and divergence
// are FP64 (fp64), FP32 (mixed) or double-float pairs of FP32 (mixed_df).
// The primitives of an upload are kept (in a buffer not needed before the first step) because
// the first stage after an upload uses them as is, like the reference after initialize.
#include <cmath>
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cato_gpu.h"
#include "cato_kernels.cuh"
#include "cato_launch.cuh"
#include "cato_pbc.cuh"
#include "cato_setup.cuh"
#include "cato_source.cuh"

using namespace cato;

namespace {

struct Plan {
  int threads = 128;       // CTA width incl. halo
  int rows_per_cta = 64;   // rows marched per CTA
  int variant = 0;         // FP64 stage kernel register budget (launch_stage_one)
};

struct Stage {
  int kind;     // StageArgs::kind
  double a, b;  // combine coefficients (kind 1 / mixed b)
  double coef;  // c = coef * dt
};

}  // namespace

struct cato_handle {
  cato_config cfg{};
  int ni = 0, nj = 0, ng = 2, pitch = 0;
  size_t field_elems = 0;
  // a slab with CATO_BC_EXCHANGE sides: U, S and the uploaded primitives hold ng ghost rows
  // below row 0 and above row nj - 1 (the buffers start row_off elements before U[v] etc.)
  bool exchange = false;
  size_t row_off = 0;
  int next_stage = -1;  // stage-by-stage step in progress: the next stage; -1 = none
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // device buffers
  double* U[4] = {};       // U^n
  double* S[2][4] = {};    // stage buffers
  double* prim_raw[4] = {};  // primitives of the last upload (alias of a free buffer)
  double* scratch[8] = {};   // solve / download / interpolation scratch (lazy)
  double* halo[4] = {};      // halo-padded scratch (lazy)
  size_t halo_elems = 0;
  StepCtl* ctl = nullptr;    // device
  StepCtl* ctl_host = nullptr;  // pinned mirror
  bool uploaded = false;
  bool raw_pending = false;  // next stage 1 uses prim_raw
  bool stepped = false;      // a step ran since the last upload (its stage buffers are valid)
  // step options (cato_gpu_set_step_options): keep U^n of each step (U_0 of the convergence
  // norms of rk(m,n) steps), and subcycle SSP steps (retry with dt / 10)
  bool keep_start = false;
  bool subcycle = false;
  double subcycle_tol = 1e-3;
  double* bak[4] = {};       // U^n of the last step
  double* bak_raw[4] = {};   // the uploaded primitives while a first step may be retried
  bool bak_valid = false;
  double* rect[6] = {};      // rectilinear grid: dx, lx, 1/dx per column; dy, ly, 1/dy per row
  float* rectf[2] = {};      // FP32 1/dx per column, 1/dy per row
  double* red = nullptr;     // reduction partials + results (lazy)
  // +x pressure input: per-row edge states + the column maximum (lazy), the target table
  double* pbc = nullptr;
  double* pbc_tab = nullptr;
  int pbc_n = 0, pbc_cap = 0;
  // rectilinear grid nodes x(1..ni+1), y(1..nj+1) (while rect_on)
  double* nodes[2] = {};
  bool rect_on = false;
  // energy source term: configuration, table (time, value, critical density), field, slots
  bool src_on = false;
  cato_energy_source src{};
  double* src_tab = nullptr;
  int src_n = 0;
  double src_tmax = 0.0;
  double* src_field = nullptr;
  int* src_dep = nullptr;
  int src_parity = 0;
  Plan plan;
  FluxConsts<double> K64{};
  FluxConsts<float> K32{};
  FluxConsts<df> Kdf{};
  Geom G{};
  std::vector<Stage> stages;
  std::string err;
  cudaStream_t own_stream_saved = nullptr;
  cudaEvent_t* event_hook = nullptr;  // profile_step: event k+1 recorded after kernel k
};

static thread_local std::string g_null_err;

static int fail(cato_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

static int cuda_fail(cato_handle* h, cudaError_t e, const char* where) {
  return fail(h, CATO_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                        \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return cuda_fail(h, _e, #call); \
  } while (0)

static int recon_of(int limiter) { return recon_of_limiter(limiter); }

// rk(m,n) stage weights, mod_fluid.f90:926-945
static const double* rk_alpha(int rk, int* ns) {
  static const double a13[] = {0.1481, 0.4, 1.0}, a14[] = {0.0833, 0.2069, 0.4265, 1.0},
                      a15[] = {0.0533, 0.1263, 0.2375, 0.4414, 1.0},
                      a23[] = {0.1918, 0.4929, 1.0}, a24[] = {0.1084, 0.2602, 0.5052, 1.0},
                      a25[] = {0.0695, 0.1602, 0.2898, 0.5060, 1.0};
  switch (rk) {
    case CATO_RK_1_3: *ns = 3; return a13;
    case CATO_RK_1_4: *ns = 4; return a14;
    case CATO_RK_1_5: *ns = 5; return a15;
    case CATO_RK_2_3: *ns = 3; return a23;
    case CATO_RK_2_4: *ns = 4; return a24;
    default: *ns = 5; return a25;
  }
}

// The stage sequence of each integrator (mod_fluid.f90:739-1160).
static std::vector<Stage> build_stages(int rk) {
  std::vector<Stage> s;
  if (rk == CATO_RK_SSP2) {
    s.push_back({0, 1.0, 0.0, 1.0});            // U1 = U + L(U)*dt
    s.push_back({1, 0.5, 0.5, 0.5});            // U2 = U*0.5 + U1*0.5 + L(U1)*(0.5*dt)
  } else if (rk == CATO_RK_SSP3) {
    s.push_back({0, 1.0, 0.0, 1.0});
    s.push_back({1, 3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0});
    s.push_back({1, 1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0});
  } else {
    int ns;
    const double* al = rk_alpha(rk, &ns);
    for (int m = 0; m < ns; ++m) s.push_back({0, 1.0, 0.0, al[m]});  // U0 + L(Uprev)*(dt*alpha)
  }
  return s;
}

static void fill_consts(cato_handle* h) {
  const FluxConsts<double> K = flux_consts_of(h->cfg);
  h->K64 = K;
  h->K32 = convert_consts<float>(K);
  h->Kdf = convert_consts<df>(K);
  h->G = uniform_geom(h->cfg.dx, h->cfg.dy);
}

static void default_plan(cato_handle* h) {
  const LaunchShape d = default_shape(h->ni, h->nj, h->ng);
  Plan p;
  p.threads = d.threads;
  p.rows_per_cta = d.rows_per_cta;
  h->plan = p;
}

static StageArgs base_args(cato_handle* h) {
  StageArgs A;
  std::memset(&A, 0, sizeof(A));
  A.ni = h->ni;
  A.nj = h->nj;
  A.pitch = h->pitch;
  for (int s = 0; s < 4; ++s) A.bc[s] = h->cfg.bc[s];
  A.limiter = h->cfg.limiter;
  A.rows_per_cta = h->plan.rows_per_cta;
  A.dt = &h->ctl->dt;
  A.active = &h->ctl->active;
  A.dt_min = &h->ctl->dt_min;
  A.status = &h->ctl->status;
  A.gamma = h->cfg.gamma;
  A.bc_p = h->cfg.bc_pressure;
  A.cfl = h->cfg.cfl;
  A.G = h->G;
  return A;
}

static cudaError_t launch(cato_handle* h, const StageArgs& A) {
  const int T = h->plan.threads;
  const int W = T - 2 * h->ng;
  dim3 grid((h->ni + W - 1) / W, (h->nj + A.rows_per_cta - 1) / A.rows_per_cta);
  const int recon = recon_of(h->cfg.limiter);
  if (h->cfg.precision == CATO_FP64)
    return launch_stage<double>(h->cfg.flux, recon, grid, T, h->stream, A, h->K64,
                                h->plan.variant);
  if (h->cfg.precision == CATO_MIXED_DF)
    return launch_stage<df>(h->cfg.flux, recon, grid, T, h->stream, A, h->Kdf);
  return launch_stage<float>(h->cfg.flux, recon, grid, T, h->stream, A, h->K32);
}

static bool has_pbc(const cato_handle* h) {
  return h->cfg.bc[CATO_PLUS_X] == CATO_BC_PRESSURE_INPUT;
}

// The pressure-input target must be usable before a step: a table, or the constant pressure
// and density of the configuration (get_desired_pressure / get_desired_density stop the
// reference on values below tiny, pressure_input_bc.f90:211-253).
static int pbc_prepare(cato_handle* h) {
  if (!has_pbc(h)) return CATO_OK;
  const double tiny = 2.2250738585072014e-308;
  if (h->pbc_n == 0 && !(h->cfg.bc_pressure >= tiny && h->cfg.bc_density >= tiny))
    return fail(h, CATO_ERR_CONFIG,
                "pressure_input: bc_pressure and bc_density must be >= tiny without a table");
  if (!h->pbc) {
    const size_t n = 3 * (size_t)(h->nj + 2 * h->ng) + 1;
    CK(cudaMalloc(&h->pbc, n * sizeof(double)));
    CK(cudaMemsetAsync(h->pbc, 0, n * sizeof(double), h->stream));
  }
  return CATO_OK;
}

// The two boundary kernels before a stage.  The boundary time of a stage is its flux solver's
// time: t_n + dt (the step control has already advanced the time), except for the first stage
// of an rk(m,n) step (rk_first), whose solver is a copy of the persistent fluid's and keeps its
// creation time: t_create + dt.
static int enqueue_pbc(cato_handle* h, StageArgs& A, bool rk_first) {
  if (!has_pbc(h)) return CATO_OK;
  PbcArgs P{};
  P.table.n = h->pbc_n;
  P.table.t = h->pbc_tab;
  P.table.p = h->pbc_tab ? h->pbc_tab + h->pbc_n : nullptr;
  P.table.rho = h->pbc_tab ? h->pbc_tab + 2 * h->pbc_n : nullptr;
  P.table.p_const = h->cfg.bc_pressure;
  P.table.rho_const = h->cfg.bc_density;
  P.edge = h->pbc;
  P.max_p = h->pbc + 3 * (size_t)(h->nj + 2 * h->ng);
  P.ctl = h->ctl;
  P.t_mode = rk_first ? 1 : 0;
  P.ng = h->ng;
  A.pbc_edge = h->pbc;
  A.pbc_ng = h->ng;
  CK(launch_pbc(h->cfg.precision, A, P, h->stream));
  return CATO_OK;
}

static int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 32) b = 152LL * 32;
  return (int)(b < 1 ? 1 : b);
}

// The energy source field of the step (source_t%integrate at the step start, once per step as
// in every integrator, e.g. ssp_rk_3_3 mod_fluid.f90:770): the deposition column (only the
// geometries that use it) and q_dot_h.
static int enqueue_source(cato_handle* h) {
  if (!h->src_on) return CATO_OK;
  SourceArgs S{};
  S.geometry = h->src.geometry;
  S.order = h->src.gaussian_order;
  S.n = h->src_n;
  S.t = h->src_tab;
  S.q = h->src_tab ? h->src_tab + h->src_n : nullptr;
  S.rho_crit = h->src_tab ? h->src_tab + 2 * h->src_n : nullptr;
  S.t_max = h->src_tmax;
  S.constant_value = h->src.constant_value;
  S.multiplier = h->src.multiplier;
  S.xlo = h->src.xlo;
  S.xhi = h->src.xhi;
  S.ylo = h->src.ylo;
  S.yhi = h->src.yhi;
  S.fwhm_x = h->src.fwhm_x;
  S.xn = h->rect_on ? h->nodes[0] : nullptr;
  S.yn = h->rect_on ? h->nodes[1] : nullptr;
  S.dx = h->cfg.dx;
  S.dy = h->cfg.dy;
  S.ni = h->ni;
  S.nj = h->nj;
  S.pitch = h->pitch;
  S.rho = h->U[0];
  S.field = h->src_field;
  S.i_dep = h->src_dep;
  S.parity = h->src_parity;
  S.ctl = h->ctl;
  const int blocks = grid_for((long long)h->ni * h->nj);
  if (S.geometry == SRC_GAUSSIAN_1D || S.geometry == SRC_DECAY) {
    source_deposit_kernel<<<blocks, 256, 0, h->stream>>>(S);
    CK(cudaGetLastError());
  }
  source_field_kernel<<<blocks, 256, 0, h->stream>>>(S);
  CK(cudaGetLastError());
  h->src_parity = 1 - h->src_parity;
  return CATO_OK;
}

// Enqueue one full time step (step control + every stage) on the handle's stream.
// The step-control kernel and the step's energy source field.
static int enqueue_step_begin(cato_handle* h) {
  step_begin_kernel<<<1, 1, 0, h->stream>>>(h->ctl);
  CK(cudaGetLastError());
  {
    const int rcs = enqueue_source(h);
    if (rcs) return rcs;
  }
  if (h->event_hook) CK(cudaEventRecord(h->event_hook[1], h->stream));
  return CATO_OK;
}

// The stencil operand of stage k: the uploaded primitives or U^n for the first stage, else the
// previous stage's output.
static double* const* stage_input(cato_handle* h, int k) {
  if (k == 0) return h->raw_pending ? h->prim_raw : h->U;
  return h->S[(k - 1) & 1];
}

// RK stage k of the step.
static int enqueue_stage(cato_handle* h, int k) {
  const int ns = (int)h->stages.size();
  const Stage& st = h->stages[k];
  StageArgs A = base_args(h);
  A.kind = st.kind;
  A.a = st.a;
  A.b = st.b;
  A.coef = st.coef;
  A.last = (k == ns - 1);
  const bool raw = (k == 0) && h->raw_pending;
  double** Un = h->U;
  double** prev = (k == 0) ? Un : h->S[(k - 1) & 1];
  double** out = A.last ? Un : h->S[k & 1];
  for (int v = 0; v < 4; ++v) {
    A.Uk[v] = prev[v];
    A.Ua[v] = Un[v];
    A.Uo[v] = out[v];
    A.Pin[v] = raw ? h->prim_raw[v] : nullptr;
  }
  A.src_q = h->src_on ? h->src_field : nullptr;
  const int rcb = enqueue_pbc(h, A, k == 0 && h->cfg.rk >= CATO_RK_1_3);
  if (rcb) return rcb;
  CK(launch(h, A));
  if (h->event_hook) CK(cudaEventRecord(h->event_hook[k + 2], h->stream));
  return CATO_OK;
}

static int enqueue_step(cato_handle* h) {
  int rc = enqueue_step_begin(h);
  if (rc) return rc;
  const int ns = (int)h->stages.size();
  for (int k = 0; k < ns; ++k) {
    rc = enqueue_stage(h, k);
    if (rc) return rc;
  }
  h->raw_pending = false;
  return CATO_OK;
}

// Entry points that step a handle on their own cannot refresh a slab's ghost rows between
// stages.
static int refuse_exchange(cato_handle* h, const char* what) {
  return fail(h, CATO_ERR_CONFIG,
              std::string(what) +
                  ": a slab with exchange sides steps through cato_gpu_step_begin/stage/end");
}

static int pull_ctl(cato_handle* h) {
  CK(cudaMemcpyAsync(h->ctl_host, h->ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CATO_OK;
}

// The reference's order of checks after a step: the pressure-input BC stops inside the boundary
// condition, before the state is checked; every stage assignment runs check_for_nans on rho, u,
// v, p (assign_fluid, mod_fluid.f90:718-721) before sanity_check looks for negative density,
// then negative pressure (:726-737).
static int status_code(int bits) {
  if (bits & ST_BC_INPUT) return CATO_ERR_BC_INPUT;
  if (bits & ST_NAN) return CATO_NANS_FOUND;
  if (bits & ST_NEG_DENSITY) return CATO_NEG_DENSITY;
  if (bits & ST_NEG_PRESSURE) return CATO_NEG_PRESSURE;
  return CATO_OK;
}

// The checks of an uploaded state (initialize_from_hdf5, mod_fluid.f90:352-360): pressure below
// tiny, then density below tiny.  A NaN (which minval skips) is not refused here: the state
// keeps its status bit, and the first step reports NANS_FOUND as the reference's first stage
// assignment does.
static int upload_code(int bits) {
  if (bits & ST_NEG_PRESSURE) return CATO_NEG_PRESSURE;
  if (bits & ST_NEG_DENSITY) return CATO_NEG_DENSITY;
  return CATO_OK;
}

static double host_decode(unsigned long long b) {
  if (b == ~0ULL) return INFINITY;
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
}

static int ensure_scratch(cato_handle* h) {
  if (h->scratch[0]) return CATO_OK;
  for (int k = 0; k < 8; ++k) CK(cudaMalloc(&h->scratch[k], h->field_elems * sizeof(double)));
  return CATO_OK;
}

static int ensure_halo(cato_handle* h) {
  if (h->halo[0]) return CATO_OK;
  h->halo_elems = (size_t)(h->ni + 2 * h->ng) * (h->nj + 2 * h->ng);
  for (int k = 0; k < 4; ++k) CK(cudaMalloc(&h->halo[k], h->halo_elems * sizeof(double)));
  return CATO_OK;
}

// host halo-padded (ld) <-> device interior (pitch)
static int h2d_interior(cato_handle* h, double* dst, const double* src, int64_t ld) {
  const double* first = src + (size_t)h->ng * ld + h->ng;
  CK(cudaMemcpy2DAsync(dst, (size_t)h->pitch * sizeof(double), first, (size_t)ld * sizeof(double),
                       (size_t)h->ni * sizeof(double), (size_t)h->nj, cudaMemcpyHostToDevice,
                       h->stream));
  return CATO_OK;
}

static int d2h_interior(cato_handle* h, double* dst, const double* src, int64_t ld) {
  double* first = dst + (size_t)h->ng * ld + h->ng;
  CK(cudaMemcpy2DAsync(first, (size_t)ld * sizeof(double), src, (size_t)h->pitch * sizeof(double),
                       (size_t)h->ni * sizeof(double), (size_t)h->nj, cudaMemcpyDeviceToHost,
                       h->stream));
  return CATO_OK;
}

// zero the ghost ring of a halo-padded host field (the interior is overwritten by the copy that
// follows): the first and last ng columns in full, ng cells at both ends of every other column
static void zero_host_field(cato_handle* h, double* a, int64_t ld) {
  const size_t ng = (size_t)h->ng, ni = (size_t)h->ni, nj = (size_t)h->nj;
  const size_t len = ni + 2 * ng;
  for (size_t j = 0; j < nj + 2 * ng; ++j) {
    double* col = a + j * ld;
    if (j < ng || j >= nj + ng) {
      std::memset(col, 0, sizeof(double) * len);
    } else {
      std::memset(col, 0, sizeof(double) * ng);
      std::memset(col + ng + ni, 0, sizeof(double) * ng);
    }
  }
}


// cato_gpu_check_divsqrt: seeded operands through the integer-pipe division and square root of
// the FP64 path and through the hardware instructions.  Families (by the top bits of the first
// hash): random bit patterns (all classes, incl. zeros, subnormals, inf, NaN), a of a narrow
// exponent range over b in [1, 2), b with few significand bits, a close to b.  c[0]/c[2] count
// the cases the integer routines took, c[1]/c[3] their mismatches.
static __device__ __forceinline__ unsigned long long check_mix(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
static __global__ void divsqrt_check_kernel(long long n, unsigned long long seed,
                                            unsigned long long* c) {
  unsigned long long nd = 0, bd = 0, ns = 0, bs = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long h1 = check_mix(seed + 2 * (unsigned long long)i);
    const unsigned long long h2 = check_mix(seed + 2 * (unsigned long long)i + 1);
    unsigned long long ua = h1, ub = h2;
    const int fam = (int)(h1 >> 62);
    if (fam == 1) {
      ua = (ua & ~(0x7ffULL << 52)) | ((unsigned long long)(990 + (h2 & 63)) << 52);
      ub = (ub & ~(0x7ffULL << 52)) | (1023ULL << 52);
    } else if (fam == 2) {
      ub &= ~0xfffffffffff00ULL;
    } else if (fam == 3) {
      ua = (ub & 0xfffffffffffff000ULL) | (h1 & 0xfffULL);
    }
    const double a = __longlong_as_double((long long)ua), b = __longlong_as_double((long long)ub);
    bool ok;
    const uint64_t q = intdiv::div_bits(ua, ub, ok);
    if (ok) {
      ++nd;
      bd += q != (uint64_t)__double_as_longlong(a / b);
    }
    const unsigned long long us = ua & 0x7fffffffffffffffULL;
    const uint64_t r = intdiv::sqrt_bits(us, ok);
    if (ok) {
      ++ns;
      bs += r != (uint64_t)__double_as_longlong(sqrt(__longlong_as_double((long long)us)));
    }
  }
  atomicAdd(c + 0, nd);
  atomicAdd(c + 1, bd);
  atomicAdd(c + 2, ns);
  atomicAdd(c + 3, bs);
}

// The FP32 seeds of the integer routines over every input they take: the 2^23 truncated divisor
// significands fb in [1, 2) and the 2^24 square-root operands fa in [1, 4).  u[0] / u[1]: the
// largest distance, in units in the last place, of the hardware reciprocal / reciprocal square
// root approximation from the correctly rounded FP32 value (for 1/sqrt: RN32 of the FP64 value
// 1 / sqrt(fa), the host test's reference).
static __global__ void seed_ulps_kernel(unsigned* u) {
  const unsigned n = (1u << 23) + (1u << 24);
  unsigned m0 = 0, m1 = 0;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (i < (1u << 23)) {
      const float fb = __uint_as_float(0x3f800000u | i);
      const int d = (int)__float_as_uint(intdiv::recip_seed(fb)) - (int)__float_as_uint(__frcp_rn(fb));
      m0 = max(m0, (unsigned)abs(d));
    } else {
      const unsigned j = i - (1u << 23);
      const float fa = __uint_as_float(((127u + (j >> 23)) << 23) | (j & 0x7fffffu));
      const float ref = __double2float_rn(1.0 / sqrt((double)fa));
      const int d = (int)__float_as_uint(intdiv::rsqrt_seed(fa)) - (int)__float_as_uint(ref);
      m1 = max(m1, (unsigned)abs(d));
    }
  }
  atomicMax(u + 0, m0);
  atomicMax(u + 1, m1);
}

extern "C" {

const char* cato_gpu_version(void) { return "cato-gb300 0.1 (sm_103a)"; }

int cato_config_default(cato_config* c, int32_t ni, int32_t nj) {
  if (!c) return CATO_ERR_ARG;
  std::memset(c, 0, sizeof(*c));
  // mod_input.f90:34-148 defaults
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

int cato_config_check(const cato_config* c) {
  if (!c) return CATO_ERR_ARG;
  if (c->ni < 1 || c->nj < 1) return CATO_ERR_CONFIG;
  if (c->flux < CATO_FLUX_AUSMPW_PLUS || c->flux > CATO_FLUX_M_AUSMPW_PLUS) return CATO_ERR_CONFIG;
  if (c->limiter < CATO_LIM_MINMOD || c->limiter > CATO_LIM_MLP5) return CATO_ERR_CONFIG;
  if (c->rk < CATO_RK_SSP2 || c->rk > CATO_RK_2_5) return CATO_ERR_CONFIG;
  const int need = (c->limiter == CATO_LIM_MLP5) ? 3 : 2;  // mod_input.f90:320-338
  if (c->n_ghost != need) return CATO_ERR_CONFIG;
  if (c->ni < c->n_ghost || c->nj < c->n_ghost) return CATO_ERR_CONFIG;
  bool outlet = false, exchange = false, pinput = false;
  for (int s = 0; s < 4; ++s) {
    if (c->bc[s] < CATO_BC_ZERO_GRADIENT || c->bc[s] > CATO_BC_EXCHANGE) return CATO_ERR_CONFIG;
    outlet |= c->bc[s] == CATO_BC_OUTLET;
    // apply_pressure_input_primitive_var_bc only implements +x (pressure_input_bc.f90:404-409)
    if (c->bc[s] == CATO_BC_PRESSURE_INPUT && s != CATO_PLUS_X) return CATO_ERR_CONFIG;
    pinput |= c->bc[s] == CATO_BC_PRESSURE_INPUT;
    // slabs are cut along j only
    if (c->bc[s] == CATO_BC_EXCHANGE && s != CATO_PLUS_Y && s != CATO_MINUS_Y)
      return CATO_ERR_CONFIG;
    exchange |= c->bc[s] == CATO_BC_EXCHANGE;
  }
  // the pressure-input state uses the maximum pressure of the whole boundary column
  // (pressure_input_bc.f90:300-312), which a slab does not hold
  if (exchange && pinput) return CATO_ERR_CONFIG;
  // outlet_bc_constructor stops on an ambient pressure <= 0 (outlet_bc.f90:54-59)
  if (outlet && !(c->bc_pressure > 0.0)) return CATO_ERR_CONFIG;
  // periodic must be paired on an axis: an unpaired periodic side leaves ghost corners unset
  if ((c->bc[CATO_PLUS_X] == CATO_BC_PERIODIC) != (c->bc[CATO_MINUS_X] == CATO_BC_PERIODIC))
    return CATO_ERR_CONFIG;
  if ((c->bc[CATO_PLUS_Y] == CATO_BC_PERIODIC) != (c->bc[CATO_MINUS_Y] == CATO_BC_PERIODIC))
    return CATO_ERR_CONFIG;
  if (!(c->gamma > 1.0) || !(c->cfl > 0.0) || !(c->dx > 0.0) || !(c->dy > 0.0))
    return CATO_ERR_CONFIG;
  if (c->precision != CATO_FP64 && c->precision != CATO_MIXED && c->precision != CATO_MIXED_DF)
    return CATO_ERR_CONFIG;
  if (c->roe_entropy_fix != CATO_ROE_REFERENCE && c->roe_entropy_fix != CATO_ROE_HARTEN)
    return CATO_ERR_CONFIG;
  if ((long long)c->ni > (1LL << 30) || (long long)c->nj > (1LL << 30)) return CATO_ERR_CONFIG;
  return CATO_OK;
}

int cato_gpu_create(const cato_config* cfg, cato_handle** out) {
  if (!cfg || !out) return CATO_ERR_ARG;
  *out = nullptr;
  int rc = cato_config_check(cfg);
  if (rc != CATO_OK) return rc;
  cato_handle* h = new cato_handle();
  h->cfg = *cfg;
  h->ni = cfg->ni;
  h->nj = cfg->nj;
  h->ng = cfg->n_ghost;
  h->pitch = (cfg->ni + 31) / 32 * 32;
  h->field_elems = (size_t)h->pitch * h->nj;
  h->exchange = cfg->bc[CATO_PLUS_Y] == CATO_BC_EXCHANGE || cfg->bc[CATO_MINUS_Y] == CATO_BC_EXCHANGE;
  h->row_off = h->exchange ? (size_t)h->ng * h->pitch : 0;
  h->stages = build_stages(cfg->rk);
  fill_consts(h);
  default_plan(h);
  auto cleanup = [&](int code) {
    cato_gpu_destroy(h);
    return code;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete h; return CATO_ERR_CUDA; }
  h->own_stream = true;
  // the state buffers, with the ghost rows of the exchange sides around them
  const size_t fb = (h->field_elems + 2 * h->row_off) * sizeof(double);
  auto dalloc = [&](double** p, size_t bytes) -> bool {
    void* q = nullptr;
    cudaError_t ee = cudaMalloc(&q, bytes);
    if (ee != cudaSuccess) { (void)cudaGetLastError(); return false; }
    *p = static_cast<double*>(q) + h->row_off;
    return true;
  };
  for (int v = 0; v < 4; ++v) {
    if (!dalloc(&h->U[v], fb)) return cleanup(CATO_ERR_OOM);
    if (!dalloc(&h->S[0][v], fb)) return cleanup(CATO_ERR_OOM);
    if (!dalloc(&h->S[1][v], fb)) return cleanup(CATO_ERR_OOM);
    h->prim_raw[v] = h->S[1][v];  // S1 is first written by stage 2, after stage 1 read these
  }
  if (cudaMalloc((void**)&h->ctl, sizeof(StepCtl)) != cudaSuccess) {
    (void)cudaGetLastError();
    return cleanup(CATO_ERR_OOM);
  }
  if (cudaMallocHost((void**)&h->ctl_host, sizeof(StepCtl)) != cudaSuccess) return cleanup(CATO_ERR_OOM);
  std::memset(h->ctl_host, 0, sizeof(StepCtl));
  h->ctl_host->dt_min = ~0ULL;
  h->ctl_host->t_end = INFINITY;
  h->ctl_host->max_iter = (1LL << 62);
  if (cudaMemcpy(h->ctl, h->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice) != cudaSuccess)
    return cleanup(CATO_ERR_CUDA);
  // prepare the kernel's shared-memory attribute outside any stream capture
  StageArgs A = base_args(h);
  const int rc0 = recon_of(cfg->limiter);
  cudaError_t ee =
      cfg->precision == CATO_FP64
          ? launch_stage<double>(cfg->flux, rc0, dim3(0, 0), 64, h->stream, A, h->K64)
      : cfg->precision == CATO_MIXED_DF
          ? launch_stage<df>(cfg->flux, rc0, dim3(0, 0), 64, h->stream, A, h->Kdf)
          : launch_stage<float>(cfg->flux, rc0, dim3(0, 0), 64, h->stream, A, h->K32);
  if (ee != cudaSuccess) return cleanup(CATO_ERR_CUDA);
  *out = h;
  return CATO_OK;
}

int cato_gpu_destroy(cato_handle* h) {
  if (!h) return CATO_ERR_ARG;
  if (h->stream) cudaStreamSynchronize(h->stream);
  auto base = [&](double* p) { return p ? p - h->row_off : nullptr; };
  for (int v = 0; v < 4; ++v) {
    cudaFree(base(h->U[v]));
    for (int s = 0; s < 2; ++s) cudaFree(base(h->S[s][v]));
    cudaFree(h->bak[v]);
    cudaFree(h->bak_raw[v]);
  }
  for (int k = 0; k < 8; ++k) cudaFree(h->scratch[k]);
  for (int k = 0; k < 4; ++k) cudaFree(h->halo[k]);
  cudaFree(h->ctl);
  cudaFree(h->red);
  cudaFree(h->pbc);
  cudaFree(h->pbc_tab);
  for (int k = 0; k < 2; ++k) cudaFree(h->nodes[k]);
  cudaFree(h->src_tab);
  cudaFree(h->src_field);
  cudaFree(h->src_dep);
  for (int k = 0; k < 6; ++k) cudaFree(h->rect[k]);
  for (int k = 0; k < 2; ++k) cudaFree(h->rectf[k]);
  if (h->ctl_host) cudaFreeHost(h->ctl_host);
  if (h->own_stream_saved) h->stream = h->own_stream_saved;
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return CATO_OK;
}

const char* cato_gpu_last_error(const cato_handle* h) {
  return h ? h->err.c_str() : g_null_err.c_str();
}

int cato_gpu_upload_primitive(cato_handle* h, const double* rho, const double* u, const double* v,
                              const double* p, int64_t ld) {
  if (!h) return CATO_ERR_ARG;
  if (!rho || !u || !v || !p) return fail(h, CATO_ERR_ARG, "null field pointer");
  if (ld < h->ni + 2 * h->ng) return fail(h, CATO_ERR_ARG, "leading dimension too small");
  const double* src[4] = {rho, u, v, p};
  for (int k = 0; k < 4; ++k) {
    int rc = h2d_interior(h, h->prim_raw[k], src[k], ld);
    if (rc) return rc;
  }
  // a slab's ghost rows beyond its exchange sides: the neighbouring slabs' rows of the same state
  for (int side : {CATO_MINUS_Y, CATO_PLUS_Y}) {
    if (h->cfg.bc[side] != CATO_BC_EXCHANGE) continue;
    const int j0 = side == CATO_MINUS_Y ? -h->ng : h->nj;  // first ghost row, 0-based
    for (int k = 0; k < 4; ++k) {
      const double* first = src[k] + (size_t)(j0 + h->ng) * ld + h->ng;
      CK(cudaMemcpy2DAsync(h->prim_raw[k] + (ptrdiff_t)j0 * h->pitch,
                           (size_t)h->pitch * sizeof(double), first, (size_t)ld * sizeof(double),
                           (size_t)h->ni * sizeof(double), (size_t)h->ng, cudaMemcpyHostToDevice,
                           h->stream));
    }
  }
  h->next_stage = -1;
  StepCtl c{};
  c.dt_min = ~0ULL;
  c.t_end = INFINITY;
  c.max_iter = (1LL << 62);
  *h->ctl_host = c;
  CK(cudaMemcpyAsync(h->ctl, h->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice, h->stream));
  double** Un = h->U;
  upload_init_kernel<<<grid_for((long long)h->ni * h->nj), 256, 0, h->stream>>>(
      h->ni, h->nj, h->pitch, h->cfg.gamma, h->cfg.cfl, h->G.dx, h->G.dy, h->G.dxc, h->G.dyc,
      h->prim_raw[0],
      h->prim_raw[1], h->prim_raw[2], h->prim_raw[3], Un[0], Un[1], Un[2], Un[3], h->ctl);
  CK(cudaGetLastError());
  int rc = pull_ctl(h);
  if (rc) return rc;
  h->uploaded = true;
  h->bak_valid = false;
  h->raw_pending = true;
  h->stepped = false;
  return upload_code(h->ctl_host->status);
}

int cato_gpu_get_timestep(cato_handle* h, double* dt) {
  if (!h || !dt) return CATO_ERR_ARG;
  if (!h->uploaded) return fail(h, CATO_ERR_STATE, "no state uploaded");
  int rc = pull_ctl(h);
  if (rc) return rc;
  *dt = host_decode(h->ctl_host->dt_min);
  return CATO_OK;
}

// One step with the step options on: U^n (and, while the first step after an upload may be
// retried, the uploaded primitives) is copied aside first; with subcycling, an SSP step whose
// convergence norm exceeds the tolerance is undone and taken again with dt / 10
// (subcycle_check, mod_fluid.f90:856-887, inside the stage loops of ssp_rk_2_2 and ssp_rk_3_3).
static int step_kept(cato_handle* h, const StepCtl& c0) {
  const size_t fb = h->field_elems * sizeof(double);
  const int rk = h->cfg.rk;
  const bool retry = h->subcycle && (rk == CATO_RK_SSP2 || rk == CATO_RK_SSP3);
  const bool raw = h->raw_pending;
  for (int k = 0; k < 4; ++k) {
    if (!h->bak[k]) CK(cudaMalloc(&h->bak[k], fb));
    CK(cudaMemcpyAsync(h->bak[k], h->U[k], fb, cudaMemcpyDeviceToDevice, h->stream));
    if (retry && raw) {
      if (!h->bak_raw[k]) CK(cudaMalloc(&h->bak_raw[k], fb));
      CK(cudaMemcpyAsync(h->bak_raw[k], h->prim_raw[k], fb, cudaMemcpyDeviceToDevice,
                         h->stream));
    }
  }
  // the step's dt: the caller's, else the CFL dt of U^n (the step kernel's own choice)
  double dt = c0.fixed_dt > 0.0 ? c0.fixed_dt : host_decode(c0.dt_min);
  for (int attempt = 0;; ++attempt) {
    StepCtl c = c0;
    if (attempt > 0) c.fixed_dt = dt;
    *h->ctl_host = c;
    CK(cudaMemcpyAsync(h->ctl, h->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice, h->stream));
    int rc = enqueue_step(h);
    if (rc) return rc;
    rc = pull_ctl(h);
    if (rc) return rc;
    h->bak_valid = true;
    if (h->ctl_host->iter > c0.iter) h->stepped = true;
    // 40 retries take dt below 1e-40 of the CFL dt: the norm is then as small as it gets
    if (!retry || h->ctl_host->status || attempt >= 40) break;
    double l2[4];
    rc = cato_gpu_convergence(h, l2);
    if (rc) return rc;
    bool again = false;
    for (int k = 0; k < 4; ++k) again |= l2[k] > h->subcycle_tol;  // NaN: no subcycle
    if (!again) break;
    for (int k = 0; k < 4; ++k) {
      CK(cudaMemcpyAsync(h->U[k], h->bak[k], fb, cudaMemcpyDeviceToDevice, h->stream));
      if (raw)
        CK(cudaMemcpyAsync(h->prim_raw[k], h->bak_raw[k], fb, cudaMemcpyDeviceToDevice,
                           h->stream));
    }
    h->raw_pending = raw;
    dt = dt / 10.0;
  }
  return CATO_OK;
}

int cato_gpu_set_step_options(cato_handle* h, int32_t keep_step_start, int32_t allow_subcycle,
                              double subcycle_tolerance) {
  if (!h) return CATO_ERR_ARG;
  if (allow_subcycle && !(subcycle_tolerance > 0.0))
    return fail(h, CATO_ERR_ARG, "subcycle tolerance must be positive");
  // a subcycle decision needs the norms of the whole grid
  if (h->exchange && (keep_step_start || allow_subcycle))
    return fail(h, CATO_ERR_CONFIG, "step options on a slab");
  // the pressure-input boundary's clock advances with every residual evaluation in the
  // reference, so a retried step would see other boundary times: not combined here
  if (allow_subcycle && h->cfg.bc[CATO_PLUS_X] == CATO_BC_PRESSURE_INPUT)
    return fail(h, CATO_ERR_CONFIG, "subcycling with the pressure-input boundary");
  h->keep_start = keep_step_start != 0 || allow_subcycle != 0;
  h->subcycle = allow_subcycle != 0;
  h->subcycle_tol = subcycle_tolerance;
  return CATO_OK;
}

int cato_gpu_integrate(cato_handle* h, double dt, double* dt_used, int32_t* error_code) {
  if (!h) return CATO_ERR_ARG;
  if (!h->uploaded) return fail(h, CATO_ERR_STATE, "no state uploaded");
  if (h->exchange) return refuse_exchange(h, "cato_gpu_integrate");
  if (h->next_stage >= 0) return fail(h, CATO_ERR_STATE, "a stage-by-stage step is open");
  // one step regardless of t_end; fixed dt when dt > 0
  int rc = pbc_prepare(h);
  if (rc) return rc;
  rc = pull_ctl(h);
  if (rc) return rc;
  StepCtl c = *h->ctl_host;
  c.t_end = INFINITY;
  c.max_iter = c.iter + 1;
  c.fixed_dt = dt > 0.0 ? dt : 0.0;
  *h->ctl_host = c;
  if (c.status == 0 && h->keep_start) {
    rc = step_kept(h, c);
    if (rc) return rc;
  } else {
    CK(cudaMemcpyAsync(h->ctl, h->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice,
                       h->stream));
    if (c.status == 0) {
      rc = enqueue_step(h);
      if (rc) return rc;
    }
    rc = pull_ctl(h);
    if (rc) return rc;
    if (h->ctl_host->iter > c.iter) h->stepped = true;
  }
  if (dt_used) *dt_used = h->ctl_host->dt;
  if (error_code) *error_code = status_code(h->ctl_host->status);
  return CATO_OK;
}

// Stage-by-stage step (slab exchange): the kernels of enqueue_step, with the host between stages.
int cato_gpu_step_begin(cato_handle* h, double dt) {
  if (!h) return CATO_ERR_ARG;
  if (!h->uploaded) return fail(h, CATO_ERR_STATE, "no state uploaded");
  if (h->next_stage >= 0) return fail(h, CATO_ERR_STATE, "a stage-by-stage step is open");
  if (h->keep_start) return fail(h, CATO_ERR_CONFIG, "step options with stage-by-stage steps");
  int rc = pbc_prepare(h);
  if (rc) return rc;
  rc = pull_ctl(h);
  if (rc) return rc;
  StepCtl c = *h->ctl_host;
  c.t_end = INFINITY;
  c.max_iter = c.iter + 1;
  c.fixed_dt = dt > 0.0 ? dt : 0.0;
  *h->ctl_host = c;
  CK(cudaMemcpyAsync(h->ctl, h->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice, h->stream));
  // a state with an error status takes no step (the kernels see active = 0)
  rc = enqueue_step_begin(h);
  if (rc) return rc;
  h->next_stage = 0;
  return CATO_OK;
}

int cato_gpu_step_stage(cato_handle* h, int32_t* stages_left) {
  if (!h) return CATO_ERR_ARG;
  const int ns = (int)h->stages.size();
  if (h->next_stage < 0 || h->next_stage >= ns)
    return fail(h, CATO_ERR_STATE, "no stage left in this step (cato_gpu_step_begin first)");
  const int rc = enqueue_stage(h, h->next_stage);
  if (rc) return rc;
  h->next_stage += 1;
  if (stages_left) *stages_left = ns - h->next_stage;
  return CATO_OK;
}

int cato_gpu_step_end(cato_handle* h, double* dt_used, int32_t* error_code) {
  if (!h) return CATO_ERR_ARG;
  if (h->next_stage != (int)h->stages.size())
    return fail(h, CATO_ERR_STATE, "the step's stages have not all run");
  h->next_stage = -1;
  h->raw_pending = false;
  const long long it0 = h->ctl_host->iter;
  const int rc = pull_ctl(h);
  if (rc) return rc;
  if (h->ctl_host->iter > it0) h->stepped = true;
  if (dt_used) *dt_used = h->ctl_host->dt;
  if (error_code) *error_code = status_code(h->ctl_host->status);
  return CATO_OK;
}

// The next stage's input rows next to (export) or beyond (import) an exchange side.
static int halo_rows(cato_handle* h, int32_t side, double** base) {
  if (side != CATO_PLUS_Y && side != CATO_MINUS_Y) return fail(h, CATO_ERR_ARG, "side must be +-y");
  if (h->cfg.bc[side] != CATO_BC_EXCHANGE) return fail(h, CATO_ERR_ARG, "not an exchange side");
  if (!h->uploaded) return fail(h, CATO_ERR_STATE, "no state uploaded");
  const int ns = (int)h->stages.size();
  const int k = h->next_stage < 0 ? 0 : h->next_stage;
  if (k >= ns) return fail(h, CATO_ERR_STATE, "every stage of this step has run");
  double* const* in = stage_input(h, k);
  for (int v = 0; v < 4; ++v) base[v] = in[v];
  return CATO_OK;
}

int cato_gpu_halo_export(cato_handle* h, int32_t side, double* rows) {
  if (!h || !rows) return CATO_ERR_ARG;
  double* in[4];
  int rc = halo_rows(h, side, in);
  if (rc) return rc;
  const int j0 = side == CATO_MINUS_Y ? 0 : h->nj - h->ng;  // first interior row sent
  const size_t plane = (size_t)h->ng * h->ni;
  for (int v = 0; v < 4; ++v)
    CK(cudaMemcpy2DAsync(rows + v * plane, (size_t)h->ni * sizeof(double),
                         in[v] + (ptrdiff_t)j0 * h->pitch, (size_t)h->pitch * sizeof(double),
                         (size_t)h->ni * sizeof(double), (size_t)h->ng, cudaMemcpyDeviceToHost,
                         h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CATO_OK;
}

int cato_gpu_halo_import(cato_handle* h, int32_t side, const double* rows) {
  if (!h || !rows) return CATO_ERR_ARG;
  double* in[4];
  int rc = halo_rows(h, side, in);
  if (rc) return rc;
  const int j0 = side == CATO_MINUS_Y ? -h->ng : h->nj;  // first ghost row written
  const size_t plane = (size_t)h->ng * h->ni;
  for (int v = 0; v < 4; ++v)
    CK(cudaMemcpy2DAsync(in[v] + (ptrdiff_t)j0 * h->pitch, (size_t)h->pitch * sizeof(double),
                         rows + v * plane, (size_t)h->ni * sizeof(double),
                         (size_t)h->ni * sizeof(double), (size_t)h->ng, cudaMemcpyHostToDevice,
                         h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CATO_OK;
}

int cato_gpu_run(cato_handle* h, int64_t max_steps, double t_end, int64_t* steps_done,
                 double* time, int32_t* error_code) {
  if (!h) return CATO_ERR_ARG;
  if (!h->uploaded) return fail(h, CATO_ERR_STATE, "no state uploaded");
  if (h->exchange) return refuse_exchange(h, "cato_gpu_run");
  int rc = pbc_prepare(h);
  if (rc) return rc;
  rc = pull_ctl(h);
  if (rc) return rc;
  StepCtl c = *h->ctl_host;
  const long long it0 = c.iter;
  c.t_end = t_end;
  c.max_iter = max_steps >= 0 ? it0 + max_steps : (1LL << 62);
  c.fixed_dt = 0.0;
  *h->ctl_host = c;
  CK(cudaMemcpyAsync(h->ctl, h->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice, h->stream));
  const long long total = max_steps >= 0 ? max_steps : (1LL << 62);
  long long issued = 0;
  const long long chunk = 32;
  // with the step options on, each step is taken from the host (copies, subcycle decisions)
  while (h->keep_start && issued < total) {
    const StepCtl& now = *h->ctl_host;
    if (now.status != 0 || !(now.time < t_end)) break;
    StepCtl s = now;
    s.max_iter = s.iter + 1;
    s.fixed_dt = 0.0;
    rc = step_kept(h, s);
    if (rc) return rc;
    ++issued;
  }
  while (!h->keep_start && issued < total) {
    const long long n = (total - issued) < chunk ? (total - issued) : chunk;
    for (long long k = 0; k < n; ++k) {
      rc = enqueue_step(h);
      if (rc) return rc;
    }
    issued += n;
    rc = pull_ctl(h);
    if (rc) return rc;
    if (!h->ctl_host->active || h->ctl_host->status) break;
  }
  if (h->ctl_host->iter > it0) h->stepped = true;
  if (steps_done) *steps_done = h->ctl_host->iter - it0;
  if (time) *time = h->ctl_host->time;
  if (error_code) *error_code = status_code(h->ctl_host->status);
  return CATO_OK;
}

int cato_gpu_set_time(cato_handle* h, double time, int64_t iteration) {
  if (!h) return CATO_ERR_ARG;
  int rc = pull_ctl(h);
  if (rc) return rc;
  h->ctl_host->time = time;
  h->ctl_host->t_create = time;  // as a fluid created at this time (new_fluid(..., time))
  h->ctl_host->iter = iteration;
  CK(cudaMemcpyAsync(h->ctl, h->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CATO_OK;
}

int cato_gpu_get_time(cato_handle* h, double* time, int64_t* iteration, double* last_dt) {
  if (!h) return CATO_ERR_ARG;
  int rc = pull_ctl(h);
  if (rc) return rc;
  if (time) *time = h->ctl_host->time;
  if (iteration) *iteration = h->ctl_host->iter;
  if (last_dt) *last_dt = h->ctl_host->dt;
  return CATO_OK;
}

int cato_gpu_download(cato_handle* h, double* rho, double* rho_u, double* rho_v, double* rho_E,
                      double* u, double* v, double* p, double* cs, int64_t ld) {
  if (!h) return CATO_ERR_ARG;
  if (!h->uploaded) return fail(h, CATO_ERR_STATE, "no state uploaded");
  if (ld < h->ni + 2 * h->ng) return fail(h, CATO_ERR_ARG, "leading dimension too small");
  double** Un = h->U;
  double* cons_out[4] = {rho, rho_u, rho_v, rho_E};
  double* der_out[4] = {u, v, p, cs};
  int rc;
  for (int k = 0; k < 4; ++k)
    if (cons_out[k]) {
      zero_host_field(h, cons_out[k], ld);
      if ((rc = d2h_interior(h, cons_out[k], Un[k], ld))) return rc;
    }
  if (u || v || p || cs) {
    if ((rc = ensure_scratch(h))) return rc;
    const int raw = h->raw_pending ? 1 : 0;
    double* const* src = raw ? h->prim_raw : Un;
    derive_kernel<<<grid_for((long long)h->ni * h->nj), 256, 0, h->stream>>>(
        h->ni, h->nj, h->pitch, h->cfg.gamma, raw, src[0], src[1], src[2], src[3], h->scratch[0],
        h->scratch[1], h->scratch[2], h->scratch[3]);
    CK(cudaGetLastError());
    for (int k = 0; k < 4; ++k)
      if (der_out[k]) {
        zero_host_field(h, der_out[k], ld);
        if ((rc = d2h_interior(h, der_out[k], h->scratch[k], ld))) return rc;
      }
  }
  CK(cudaStreamSynchronize(h->stream));
  return CATO_OK;
}

int cato_gpu_solve(cato_handle* h, double* rho, double* u, double* v, double* p,
                   double* d_rho_dt, double* d_rho_u_dt, double* d_rho_v_dt, double* d_rho_E_dt,
                   int64_t ld) {
  if (!h) return CATO_ERR_ARG;
  if (!rho || !u || !v || !p || !d_rho_dt || !d_rho_u_dt || !d_rho_v_dt || !d_rho_E_dt)
    return fail(h, CATO_ERR_ARG, "null field pointer");
  if (ld < h->ni + 2 * h->ng) return fail(h, CATO_ERR_ARG, "leading dimension too small");
  if (h->exchange) return fail(h, CATO_ERR_CONFIG, "solve on a slab");
  int rc;
  if ((rc = pbc_prepare(h))) return rc;
  if ((rc = ensure_scratch(h))) return rc;
  if ((rc = ensure_halo(h))) return rc;
  double* prim[4] = {rho, u, v, p};
  for (int k = 0; k < 4; ++k)
    if ((rc = h2d_interior(h, h->scratch[k], prim[k], ld))) return rc;
  // residual: one stage in kind 2 reading the given primitives
  StepCtl* ctl = h->ctl;  // dt unused by kind 2; keep the handle's dt_min untouched
  (void)ctl;
  StageArgs A = base_args(h);
  A.kind = 2;
  A.last = 0;
  A.active = nullptr;
  A.coef = 0.0;
  for (int k = 0; k < 4; ++k) {
    A.Pin[k] = h->scratch[k];
    A.Uk[k] = h->scratch[k];
    A.Ua[k] = nullptr;
    A.Uo[k] = h->scratch[4 + k];
  }
  // a table target is evaluated at the handle's time (cato_gpu_set_time)
  if ((rc = enqueue_pbc(h, A, false))) return rc;
  CK(launch(h, A));
  // write the BC-filled ghosts back into the caller's primitive arrays (intent(inout))
  const int4 bc = make_int4(h->cfg.bc[0], h->cfg.bc[1], h->cfg.bc[2], h->cfg.bc[3]);
  const long long hld = h->ni + 2 * h->ng;
  fill_ghosts_kernel<<<grid_for((long long)h->halo_elems), 256, 0, h->stream>>>(
      h->ni, h->nj, h->pitch, h->ng, bc, h->cfg.gamma, h->cfg.bc_pressure, h->pbc, h->scratch[0],
      h->scratch[1], h->scratch[2], h->scratch[3], h->halo[0], h->halo[1], h->halo[2],
      h->halo[3], hld);
  CK(cudaGetLastError());
  for (int k = 0; k < 4; ++k)
    CK(cudaMemcpy2DAsync(prim[k], (size_t)ld * sizeof(double), h->halo[k], (size_t)hld * sizeof(double),
                         (size_t)hld * sizeof(double), (size_t)(h->nj + 2 * h->ng),
                         cudaMemcpyDeviceToHost, h->stream));
  double* dout[4] = {d_rho_dt, d_rho_u_dt, d_rho_v_dt, d_rho_E_dt};
  for (int k = 0; k < 4; ++k) {
    zero_host_field(h, dout[k], ld);
    if ((rc = d2h_interior(h, dout[k], h->scratch[4 + k], ld))) return rc;
  }
  CK(cudaStreamSynchronize(h->stream));
  if (has_pbc(h)) {
    if ((rc = pull_ctl(h))) return rc;
    if (h->ctl_host->status & ST_BC_INPUT)
      return fail(h, CATO_ERR_BC_INPUT, "pressure_input target below tiny at the solve time");
  }
  return CATO_OK;
}

int cato_gpu_interpolate_edges(cato_handle* h, const double* q, int64_t ld, double* i_edges,
                               double* j_edges) {
  if (!h) return CATO_ERR_ARG;
  if (!q || !i_edges || !j_edges) return fail(h, CATO_ERR_ARG, "null pointer");
  if (ld < h->ni + 2 * h->ng) return fail(h, CATO_ERR_ARG, "leading dimension too small");
  // the ghosts of a single solve come from the boundary conditions, which a slab's exchange
  // sides do not have
  if (h->exchange) return fail(h, CATO_ERR_CONFIG, "interpolate_edges on a slab");
  int rc;
  if ((rc = ensure_halo(h))) return rc;
  const long long hld = h->ni + 2 * h->ng;
  CK(cudaMemcpy2DAsync(h->halo[0], (size_t)hld * sizeof(double), q, (size_t)ld * sizeof(double),
                       (size_t)hld * sizeof(double), (size_t)(h->nj + 2 * h->ng),
                       cudaMemcpyHostToDevice, h->stream));
  const size_t nie = 2 * (size_t)(h->ni + 2) * (h->nj + 1), nje = 2 * (size_t)(h->ni + 1) * (h->nj + 2);
  double *die = nullptr, *dje = nullptr;
  CK(cudaMallocAsync(&die, nie * sizeof(double), h->stream));
  CK(cudaMallocAsync(&dje, nje * sizeof(double), h->stream));
  CK(cudaMemsetAsync(die, 0, nie * sizeof(double), h->stream));
  CK(cudaMemsetAsync(dje, 0, nje * sizeof(double), h->stream));
  const long long ne = (long long)(h->ni + 1) * (h->nj + 1);
  const int recon = recon_of(h->cfg.limiter);
  if (recon == 0)
    interp_edges_kernel<2, 0><<<grid_for(ne), 256, 0, h->stream>>>(h->ni, h->nj, h->cfg.limiter,
                                                                   h->halo[0], hld, die, dje);
  else if (recon == 3)
    interp_edges_kernel<2, 3><<<grid_for(ne), 256, 0, h->stream>>>(h->ni, h->nj, h->cfg.limiter,
                                                                   h->halo[0], hld, die, dje);
  else
    interp_edges_kernel<3, 5><<<grid_for(ne), 256, 0, h->stream>>>(h->ni, h->nj, h->cfg.limiter,
                                                                   h->halo[0], hld, die, dje);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(i_edges, die, nie * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(j_edges, dje, nje * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaFreeAsync(die, h->stream));
  CK(cudaFreeAsync(dje, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CATO_OK;
}

int cato_gpu_status(cato_handle* h, int32_t* status_bits) {
  if (!h || !status_bits) return CATO_ERR_ARG;
  int rc = pull_ctl(h);
  if (rc) return rc;
  *status_bits = h->ctl_host->status;
  return CATO_OK;
}

int cato_gpu_synchronize(cato_handle* h) {
  if (!h) return CATO_ERR_ARG;
  CK(cudaStreamSynchronize(h->stream));
  return CATO_OK;
}

int cato_gpu_set_stream(cato_handle* h, void* stream) {
  if (!h) return CATO_ERR_ARG;
  CK(cudaStreamSynchronize(h->stream));
  if (stream) {
    if (!h->own_stream_saved) h->own_stream_saved = h->stream;
    h->stream = (cudaStream_t)stream;
  } else if (h->own_stream_saved) {
    h->stream = h->own_stream_saved;
  }
  return CATO_OK;
}

int cato_gpu_run_timed(cato_handle* h, int64_t n_steps, float* total_ms, float* kernel_ms,
                       int32_t capacity) {
  if (!h || !total_ms || n_steps < 0) return CATO_ERR_ARG;
  if (!h->uploaded) return fail(h, CATO_ERR_STATE, "no state uploaded");
  if (h->exchange) return refuse_exchange(h, "cato_gpu_run_timed");
  const int nk = 1 + (int)h->stages.size();
  if (kernel_ms && capacity < nk) return fail(h, CATO_ERR_ARG, "capacity too small");
  int rc = pbc_prepare(h);
  if (rc) return rc;
  rc = pull_ctl(h);
  if (rc) return rc;
  StepCtl c = *h->ctl_host;
  const long long it0 = c.iter;
  c.t_end = INFINITY;
  c.max_iter = it0 + n_steps;
  c.fixed_dt = 0.0;
  *h->ctl_host = c;
  CK(cudaMemcpyAsync(h->ctl, h->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice, h->stream));
  // events: [start] + one after every kernel of every step
  std::vector<cudaEvent_t> ev(kernel_ms ? (size_t)n_steps * nk + 1 : 2);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  CK(cudaEventRecord(ev[0], h->stream));
  for (long long s = 0; s < n_steps; ++s) {
    if (kernel_ms) h->event_hook = ev.data() + s * nk;
    rc = enqueue_step(h);
    h->event_hook = nullptr;
    if (rc) return rc;
  }
  if (!kernel_ms) CK(cudaEventRecord(ev[1], h->stream));
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaEventElapsedTime(total_ms, ev[0], ev.back()));
  if (kernel_ms) {
    for (int k = 0; k < nk; ++k) kernel_ms[k] = 0.0f;
    for (long long s = 0; s < n_steps; ++s)
      for (int k = 0; k < nk; ++k) {
        float ms;
        CK(cudaEventElapsedTime(&ms, ev[s * nk + k], ev[s * nk + k + 1]));
        kernel_ms[k] += ms;
      }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  rc = pull_ctl(h);
  if (rc) return rc;
  if (h->ctl_host->iter > it0) h->stepped = true;
  return status_code(h->ctl_host->status);
}

int cato_gpu_set_plan(cato_handle* h, int32_t threads, int32_t rows_per_cta) {
  if (!h) return CATO_ERR_ARG;
  if (threads < 64 || threads > 256 || threads % 32 != 0 || rows_per_cta < 1 ||
      threads - 2 * h->ng < 1)
    return fail(h, CATO_ERR_ARG, "invalid plan");
  h->plan.threads = threads;
  h->plan.rows_per_cta = rows_per_cta;
  return CATO_OK;
}

int cato_gpu_set_kernel_variant(cato_handle* h, int32_t variant) {
  if (!h) return CATO_ERR_ARG;
  if (variant < 0 || variant > 2) return fail(h, CATO_ERR_ARG, "invalid kernel variant");
  h->plan.variant = variant;
  return CATO_OK;
}

int cato_gpu_get_kernel_variant(const cato_handle* h, int32_t* variant) {
  if (!h || !variant) return CATO_ERR_ARG;
  *variant = h->plan.variant;
  return CATO_OK;
}

int cato_gpu_tune(cato_handle* h, int32_t steps, int32_t* steps_taken, float* best_ms) {
  if (!h || steps < 1) return CATO_ERR_ARG;
  if (steps_taken) *steps_taken = 0;
  if (!h->uploaded) return fail(h, CATO_ERR_STATE, "no state uploaded");
  if (h->exchange) return refuse_exchange(h, "cato_gpu_tune");
  // candidates: the default plan and 256-wide strips, each with the default, half and a quarter
  // of the rows per CTA, and with every FP64 register budget
  const Plan p0 = h->plan;
  std::vector<Plan> cands;
  const int wide = 256, half_rows = std::max(8, p0.rows_per_cta / 2);
  const int quarter_rows = std::max(8, p0.rows_per_cta / 4);
  const int nvar = h->cfg.precision == CATO_FP64 ? 3 : 1;
  for (int v = 0; v < nvar; ++v) {
    Plan a = p0, b = p0, c = p0, d = p0, e = p0, f = p0;
    a.variant = b.variant = c.variant = d.variant = e.variant = f.variant = v;
    b.threads = e.threads = f.threads = wide;
    c.rows_per_cta = e.rows_per_cta = half_rows;
    d.rows_per_cta = f.rows_per_cta = quarter_rows;
    for (const Plan& q : {a, b, c, d, e, f}) {
      bool dup = false;
      for (const Plan& x : cands)
        dup |= x.threads == q.threads && x.rows_per_cta == q.rows_per_cta && x.variant == q.variant;
      if (!dup && q.threads - 2 * h->ng <= h->ni + 2 * h->ng) cands.push_back(q);
    }
  }
  Plan best = p0;
  float best_t = INFINITY;
  int taken = 0;
  for (const Plan& q : cands) {
    h->plan = q;
    float ms = 0.0f;
    const int rc = cato_gpu_run_timed(h, steps, &ms, nullptr, 0);
    taken += steps;
    if (rc) {
      h->plan = best_t < INFINITY ? best : p0;
      if (steps_taken) *steps_taken = taken;
      return rc;
    }
    if (ms < best_t) {
      best_t = ms;
      best = q;
    }
  }
  h->plan = best;
  if (steps_taken) *steps_taken = taken;
  if (best_ms) *best_ms = best_t / (float)steps;
  return CATO_OK;
}

int cato_gpu_get_plan(const cato_handle* h, int32_t* threads, int32_t* rows_per_cta) {
  if (!h) return CATO_ERR_ARG;
  if (threads) *threads = h->plan.threads;
  if (rows_per_cta) *rows_per_cta = h->plan.rows_per_cta;
  return CATO_OK;
}

int cato_gpu_select_device(int32_t device) {
  return cudaSetDevice(device) == cudaSuccess ? CATO_OK : CATO_ERR_CUDA;
}

int cato_gpu_check_divsqrt(int64_t n, uint64_t seed, uint64_t tested[2], uint64_t mismatches[2],
                           int32_t seed_ulps[2]) {
  if (n < 0 || !tested || !mismatches || !seed_ulps) return CATO_ERR_ARG;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 5 * sizeof(unsigned long long)) != cudaSuccess) return CATO_ERR_OOM;
  unsigned* du = reinterpret_cast<unsigned*>(d + 4);
  cudaError_t e = cudaMemset(d, 0, 5 * sizeof(unsigned long long));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = (unsigned)(sms > 0 ? 8 * sms : 1024);
  if (e == cudaSuccess && n > 0) {
    divsqrt_check_kernel<<<grid, 256>>>(n, seed, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    seed_ulps_kernel<<<grid, 256>>>(du);
    e = cudaGetLastError();
  }
  unsigned long long h[5] = {0, 0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  tested[0] = h[0];
  mismatches[0] = h[1];
  tested[1] = h[2];
  mismatches[1] = h[3];
  unsigned hu[2];
  memcpy(hu, &h[4], sizeof hu);
  seed_ulps[0] = (int32_t)hu[0];
  seed_ulps[1] = (int32_t)hu[1];
  return e == cudaSuccess ? CATO_OK : CATO_ERR_CUDA;
}

int cato_host_alloc(uint64_t bytes, void** out) {
  if (!out) return CATO_ERR_ARG;
  *out = nullptr;
  return cudaHostAlloc(out, bytes, cudaHostAllocPortable) == cudaSuccess ? CATO_OK : CATO_ERR_OOM;
}

int cato_host_free(void* p) { return cudaFreeHost(p) == cudaSuccess ? CATO_OK : CATO_ERR_CUDA; }

int cato_gpu_launches_per_step(const cato_handle* h, int32_t* n) {
  if (!h || !n) return CATO_ERR_ARG;
  // step control (+ the source field kernels) + per stage: the stage kernel (+ the two
  // pressure-input boundary kernels)
  const int src = !h->src_on ? 0 : (h->src.geometry == CATO_SRC_GAUSSIAN_1D ||
                                    h->src.geometry == CATO_SRC_DECAY ? 2 : 1);
  *n = 1 + src + (int32_t)h->stages.size() * (has_pbc(h) ? 3 : 1);
  return CATO_OK;
}

int cato_gpu_profile_step(cato_handle* h, float* kernel_ms, int32_t capacity, int32_t* n_kernels) {
  if (!h || !kernel_ms) return CATO_ERR_ARG;
  if (!h->uploaded) return fail(h, CATO_ERR_STATE, "no state uploaded");
  if (h->exchange) return refuse_exchange(h, "cato_gpu_profile_step");
  const int nk = 1 + (int)h->stages.size();
  if (capacity < nk) return fail(h, CATO_ERR_ARG, "capacity too small");
  int rc = pbc_prepare(h);
  if (rc) return rc;
  rc = pull_ctl(h);
  if (rc) return rc;
  StepCtl c = *h->ctl_host;
  c.t_end = INFINITY;
  c.max_iter = c.iter + 1;
  c.fixed_dt = 0.0;
  *h->ctl_host = c;
  CK(cudaMemcpyAsync(h->ctl, h->ctl_host, sizeof(StepCtl), cudaMemcpyHostToDevice, h->stream));
  std::vector<cudaEvent_t> ev(nk + 1);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  h->event_hook = ev.data();
  CK(cudaEventRecord(ev[0], h->stream));
  rc = enqueue_step(h);
  h->event_hook = nullptr;
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < nk; ++k) CK(cudaEventElapsedTime(&kernel_ms[k], ev[k], ev[k + 1]));
  for (auto& e : ev) cudaEventDestroy(e);
  if (n_kernels) *n_kernels = nk;
  rc = pull_ctl(h);
  if (rc) return rc;
  if (h->ctl_host->iter > c.iter) h->stepped = true;
  return CATO_OK;
}

int cato_gpu_set_energy_source(cato_handle* h, const cato_energy_source* src, int32_t n,
                               const double* time, const double* value,
                               const double* critical_density) {
  if (!h) return CATO_ERR_ARG;
  // the source is placed by cell centroids measured from the grid's origin, which a slab's
  // uniform geometry does not know
  if (src && h->exchange) return fail(h, CATO_ERR_CONFIG, "energy source on a slab");
  CK(cudaStreamSynchronize(h->stream));
  if (!src) {
    h->src_on = false;
    return CATO_OK;
  }
  if (src->geometry < CATO_SRC_UNIFORM || src->geometry > CATO_SRC_DECAY)
    return fail(h, CATO_ERR_CONFIG, "unsupported source geometry");
  if (src->geometry == CATO_SRC_GAUSSIAN_1D) {
    // new_source (mod_source.f90:111-119) and get_source_field (:386-388)
    if (src->gaussian_order < 1) return fail(h, CATO_ERR_CONFIG, "gaussian order < 1");
    if (!(src->fwhm_x > 0.0 && !(src->fwhm_y > 0.0)))
      return fail(h, CATO_ERR_CONFIG, "a 1d_gaussian source must be constant in y");
  }
  if (n == 1 || n < 0) return fail(h, CATO_ERR_ARG, "a table needs at least two points");
  if (n > 0) {
    if (!time || !value || !critical_density) return fail(h, CATO_ERR_ARG, "null table");
    for (int k = 0; k < n; ++k) {
      if (!std::isfinite(time[k]) || !std::isfinite(value[k]) ||
          !std::isfinite(critical_density[k]))
        return fail(h, CATO_ERR_ARG, "non-finite table entry");
      if (k > 0 && !(time[k] > time[k - 1]))
        return fail(h, CATO_ERR_ARG, "table times must be strictly increasing");
    }
    cudaFree(h->src_tab);
    h->src_tab = nullptr;
    CK(cudaMalloc(&h->src_tab, 3 * (size_t)n * sizeof(double)));
    const double* s3[3] = {time, value, critical_density};
    for (int k = 0; k < 3; ++k)
      CK(cudaMemcpy(h->src_tab + (size_t)k * n, s3[k], n * sizeof(double),
                    cudaMemcpyHostToDevice));
    h->src_tmax = time[0];
    for (int k = 1; k < n; ++k) h->src_tmax = std::max(h->src_tmax, time[k]);
  }
  if (!h->src_field) CK(cudaMalloc(&h->src_field, h->field_elems * sizeof(double)));
  if (!h->src_dep) CK(cudaMalloc(&h->src_dep, 2 * sizeof(int)));
  CK(cudaMemset(h->src_dep, 0xff, 2 * sizeof(int)));  // -1: no column found yet
  h->src_parity = 0;
  h->src = *src;
  h->src_n = n;
  h->src_on = true;
  return CATO_OK;
}

int cato_gpu_set_bc_table(cato_handle* h, int32_t n, const double* time, const double* pressure,
                          const double* density) {
  if (!h) return CATO_ERR_ARG;
  if (n == 0) {  // back to the constant target of the configuration
    h->pbc_n = 0;
    return CATO_OK;
  }
  if (!time || !pressure || !density) return fail(h, CATO_ERR_ARG, "null table pointer");
  // linear_interp_1d%initialize: at least two points, strictly increasing times (finterp
  // linear_interpolation_module.f90:451-478, 1743-1810)
  if (n < 2) return fail(h, CATO_ERR_ARG, "a table needs at least two points");
  for (int k = 0; k < n; ++k) {
    if (!std::isfinite(time[k]) || !std::isfinite(pressure[k]) || !std::isfinite(density[k]))
      return fail(h, CATO_ERR_ARG, "non-finite table entry");
    if (k > 0 && !(time[k] > time[k - 1]))
      return fail(h, CATO_ERR_ARG, "table times must be strictly increasing");
  }
  CK(cudaStreamSynchronize(h->stream));
  if (h->pbc_tab && n > h->pbc_cap) {
    CK(cudaFree(h->pbc_tab));
    h->pbc_tab = nullptr;
    h->pbc_cap = 0;
  }
  if (!h->pbc_tab) {
    CK(cudaMalloc(&h->pbc_tab, 3 * (size_t)n * sizeof(double)));
    h->pbc_cap = n;
  }
  const double* src[3] = {time, pressure, density};
  for (int k = 0; k < 3; ++k)
    CK(cudaMemcpy(h->pbc_tab + (size_t)k * n, src[k], n * sizeof(double),
                  cudaMemcpyHostToDevice));
  h->pbc_n = n;
  return CATO_OK;
}

// Per-column (or per-row) metrics of a rectilinear grid from its n + 1 nodes, with the
// quad_cell.f90 formulas on an axis-aligned cell: width x(i+1) - x(i), edge length
// sqrt(width^2 + 0^2) and the reciprocal width (FP64 and FP32).
static __global__ void rect_metrics_kernel(const double* __restrict__ nodes, int n, double* d,
                                           double* l, double* r, float* rf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double w = nodes[i + 1] - nodes[i];
    d[i] = w;
    l[i] = sqrt(w * w + 0.0 * 0.0);
    r[i] = 1.0 / w;
    rf[i] = d2f_int(1.0 / w);
  }
}

int cato_gpu_set_rectilinear(cato_handle* h, const double* x_nodes, const double* y_nodes) {
  if (!h) return CATO_ERR_ARG;
  if (!x_nodes != !y_nodes) return fail(h, CATO_ERR_ARG, "give both node arrays or neither");
  CK(cudaStreamSynchronize(h->stream));
  h->uploaded = false;  // the stored CFL dt and state were for the previous geometry
  h->stepped = false;
  if (!x_nodes) {  // back to the uniform dx x dy grid of the configuration
    h->rect_on = false;
    h->G.dxc = h->G.lxc = h->G.rdxc = h->G.dyc = h->G.lyc = h->G.rdyc = nullptr;
    h->G.rdxf = h->G.rdyf = nullptr;
    return CATO_OK;
  }
  const int n[2] = {h->ni, h->nj};
  const double* nodes[2] = {x_nodes, y_nodes};
  for (int a = 0; a < 2; ++a)
    for (int k = 0; k < n[a]; ++k)
      if (!(nodes[a][k + 1] > nodes[a][k]) || !std::isfinite(nodes[a][k + 1] - nodes[a][k]))
        return fail(h, CATO_ERR_ARG, "node coordinates must be finite and strictly increasing");
  for (int a = 0; a < 2; ++a) {
    for (int k = 0; k < 3; ++k)
      if (!h->rect[3 * a + k]) CK(cudaMalloc(&h->rect[3 * a + k], (n[a] + 1) * sizeof(double)));
    if (!h->rectf[a]) CK(cudaMalloc(&h->rectf[a], (n[a] + 1) * sizeof(float)));
  }
  for (int a = 0; a < 2; ++a) {
    // the nodes stay on the device (cell centroids of the energy source term)
    if (!h->nodes[a]) CK(cudaMalloc(&h->nodes[a], (n[a] + 1) * sizeof(double)));
    CK(cudaMemcpyAsync(h->nodes[a], nodes[a], (n[a] + 1) * sizeof(double),
                       cudaMemcpyHostToDevice, h->stream));
    rect_metrics_kernel<<<grid_for(n[a]), 256, 0, h->stream>>>(
        h->nodes[a], n[a], h->rect[3 * a], h->rect[3 * a + 1], h->rect[3 * a + 2], h->rectf[a]);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
  }
  h->rect_on = true;
  h->G.dxc = h->rect[0]; h->G.lxc = h->rect[1]; h->G.rdxc = h->rect[2]; h->G.rdxf = h->rectf[0];
  h->G.dyc = h->rect[3]; h->G.lyc = h->rect[4]; h->G.rdyc = h->rect[5]; h->G.rdyf = h->rectf[1];
  return CATO_OK;
}

static int reduce(cato_handle* h, RedArgs R, double out[RED_Q]) {
  if (!h->red) CK(cudaMalloc(&h->red, (RED_BLOCKS + 1) * RED_Q * sizeof(double)));
  R.ni = h->ni;
  R.nj = h->nj;
  R.pitch = h->pitch;
  R.partials = h->red;
  reduce_partials_kernel<<<RED_BLOCKS, RED_THREADS, 0, h->stream>>>(R);
  CK(cudaGetLastError());
  reduce_final_kernel<<<1, RED_THREADS, 0, h->stream>>>(h->red, RED_BLOCKS,
                                                       h->red + RED_BLOCKS * RED_Q);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, h->red + RED_BLOCKS * RED_Q, RED_Q * sizeof(double),
                     cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return CATO_OK;
}

// U^n of the handle
static double* const* state_now(cato_handle* h) { return h->U; }

int cato_gpu_conservation_sums(cato_handle* h, double totals[4]) {
  if (!h || !totals) return CATO_ERR_ARG;
  if (!h->uploaded) return fail(h, CATO_ERR_STATE, "no state uploaded");
  RedArgs R{};
  R.mode = 0;
  double* const* U = state_now(h);
  for (int k = 0; k < 4; ++k) R.A[k] = U[k];
  R.dxc = h->G.dxc;
  R.dyc = h->G.dyc;
  double out[RED_Q];
  int rc = reduce(h, R, out);
  if (rc) return rc;
  for (int k = 0; k < 4; ++k) totals[k] = h->G.dxc ? out[k] : out[k] * h->G.vol;
  return CATO_OK;
}

int cato_gpu_convergence(cato_handle* h, double l2[4]) {
  if (!h || !l2) return CATO_ERR_ARG;
  if (!h->uploaded || !h->stepped) return fail(h, CATO_ERR_STATE, "no step since the upload");
  const int rk = h->cfg.rk;
  const bool ssp = rk == CATO_RK_SSP2 || rk == CATO_RK_SSP3;
  RedArgs R{};
  R.mode = 1;
  // SSP: the first stage's output U_1 is still in S0.  rk(m,n) compares with U^n
  // (mod_fluid.f90:970), which the last stage overwrote in place: only a kept copy has it
  if (!ssp && !h->bak_valid)
    return fail(h, CATO_ERR_STATE,
                "rk(m,n) steps update U^n in place: keep the step start to compare with U_0");
  for (int k = 0; k < 4; ++k) {
    R.A[k] = ssp ? h->S[0][k] : h->bak[k];
    R.B[k] = h->U[k];
  }
  double out[RED_Q];
  int rc = reduce(h, R, out);
  if (rc) return rc;
  for (int k = 0; k < 4; ++k) {
    double n0 = sqrt(out[4 + k]);
    if (k == 1 || k == 2) n0 = n0 > 1.0 ? n0 : 1.0;
    l2[k] = sqrt(out[k]) / n0;
  }
  return CATO_OK;
}

}  // extern "C"
