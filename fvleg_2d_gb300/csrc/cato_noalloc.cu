// cato_noalloc.cu -- cato_gpu_solve_noalloc: the flux_solver_t%solve residual for callers that
// cannot allocate device memory.
//
// Who needs it: a caller whose device memory is owned by someone else (a framework's caching
// allocator or a fixed HBM budget, where cudaMalloc either fails or fragments the owner's pool),
// and a caller inside a latency-critical loop, where cudaMalloc / cudaFree can synchronize the
// whole device.  cato_gpu_solve needs a handle, and a handle allocates its state and scratch;
// this entry point allocates nothing.  All of its device memory is one file-scope
// `static __device__` array of fixed size, which every GPU that loads this library holds until
// the process exits.
//
// Using it:
// * Capacity: kScratchDoubles doubles (32 MiB).  A grid needs
//   8 * pitch * nj + 4 * (ni + 2 ng) * (nj + 2 ng) + 32 doubles, pitch = ni rounded up to 32;
//   e.g. 512 x 512 fits, 600 x 600 does not.  Larger grids are refused with
//   CATO_ERR_CAPACITY before any GPU work.
// * The first call on a device looks up the array's device address (cudaGetSymbolAddress, with
//   that device current) and caches it per device; make that first call before any CUDA stream
//   capture.  The cached address belongs to the device's primary context: after
//   cudaDeviceReset on that device the entry point must not be called again in this process.
// * Every call in the process shares the one array, which keeps the last call's contents.  Calls
//   that overlapped on the GPU would race on it, so each call holds a per-device lock, works on
//   the calling thread's per-thread default stream (cudaStreamPerThread, which does not wait for
//   or block the process's other streams) and synchronizes it before returning.
#include <cstring>
#include <mutex>

#include "../../include/cato_gpu.h"
#include "cato_kernels.cuh"
#include "cato_launch.cuh"
#include "cato_setup.cuh"

using namespace cato;

namespace {

constexpr size_t kScratchDoubles = size_t(4) << 20;  // 4 Mi doubles = 32 MiB per device
constexpr size_t kAlign = 32;                         // doubles (256 B)

}  // namespace

// Host code must not use this name as a device address: take it from cudaGetSymbolAddress.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

namespace {

std::mutex g_dev_mutex[kMaxDevices];
double* g_scratch_dev[kMaxDevices] = {};

size_t round_up(size_t n) { return (n + kAlign - 1) / kAlign * kAlign; }

}  // namespace

extern "C" int cato_gpu_solve_noalloc(const cato_config* cfg, double* rho, double* u, double* v,
                                      double* p, double* d_rho_dt, double* d_rho_u_dt,
                                      double* d_rho_v_dt, double* d_rho_E_dt, int64_t ld) {
  if (!cfg || !rho || !u || !v || !p || !d_rho_dt || !d_rho_u_dt || !d_rho_v_dt || !d_rho_E_dt)
    return CATO_ERR_ARG;
  int rc = cato_config_check(cfg);
  if (rc != CATO_OK) return rc;
  if (cfg->precision != CATO_FP64) return CATO_ERR_CONFIG;
  // the pressure-input boundary needs per-row device state: handle entry points only
  if (cfg->bc[CATO_PLUS_X] == CATO_BC_PRESSURE_INPUT) return CATO_ERR_CONFIG;
  // slab exchange sides have no boundary condition to fill their ghosts from
  if (cfg->bc[CATO_PLUS_Y] == CATO_BC_EXCHANGE || cfg->bc[CATO_MINUS_Y] == CATO_BC_EXCHANGE)
    return CATO_ERR_CONFIG;
  const int ni = cfg->ni, nj = cfg->nj, ng = cfg->n_ghost;
  if (ld < ni + 2 * ng) return CATO_ERR_ARG;
  const int pitch = (ni + 31) / 32 * 32;
  const size_t field = round_up((size_t)pitch * nj);
  const long long hld = ni + 2 * ng;
  const size_t halo = round_up((size_t)hld * (nj + 2 * ng));
  const size_t ctl_doubles = kAlign;  // dt, CFL-dt bits, status word
  const size_t need = 8 * field + 4 * halo + ctl_doubles;
  if (need > kScratchDoubles) return CATO_ERR_CAPACITY;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CATO_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_dev_mutex[dev]);
  if (!g_scratch_dev[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
      (void)cudaGetLastError();
      return CATO_ERR_CUDA;
    }
    g_scratch_dev[dev] = static_cast<double*>(ptr);
  }
  double* base = g_scratch_dev[dev];
  double* prim[4];
  double* res[4];
  double* gh[4];
  for (int k = 0; k < 4; ++k) {
    prim[k] = base + k * field;
    res[k] = base + (4 + k) * field;
    gh[k] = base + 8 * field + k * halo;
  }
  double* ctl = base + 8 * field + 4 * halo;
  const cudaStream_t s = cudaStreamPerThread;
  double* host_prim[4] = {rho, u, v, p};
  double* host_res[4] = {d_rho_dt, d_rho_u_dt, d_rho_v_dt, d_rho_E_dt};

#define NA_CK(call)                            \
  do {                                         \
    if ((call) != cudaSuccess) {               \
      (void)cudaGetLastError();                \
      cudaStreamSynchronize(s);                \
      return CATO_ERR_CUDA;                    \
    }                                          \
  } while (0)

  // the control block is read by the stage kernel: start it from zero on every call
  NA_CK(cudaMemsetAsync(ctl, 0, ctl_doubles * sizeof(double), s));
  for (int k = 0; k < 4; ++k)
    NA_CK(cudaMemcpy2DAsync(prim[k], (size_t)pitch * sizeof(double),
                            host_prim[k] + (size_t)ng * ld + ng, (size_t)ld * sizeof(double),
                            (size_t)ni * sizeof(double), (size_t)nj, cudaMemcpyHostToDevice, s));

  // flux constants, uniform geometry and launch shape: those a handle derives from cfg
  const FluxConsts<double> K = flux_consts_of(*cfg);
  const Geom G = uniform_geom(cfg->dx, cfg->dy);
  const LaunchShape shape = default_shape(ni, nj, ng);

  StageArgs A;
  std::memset(&A, 0, sizeof(A));
  A.ni = ni;
  A.nj = nj;
  A.pitch = pitch;
  for (int k = 0; k < 4; ++k) A.bc[k] = cfg->bc[k];
  A.limiter = cfg->limiter;
  const int threads = shape.threads;
  A.rows_per_cta = shape.rows_per_cta;
  A.kind = 2;
  A.dt = ctl;
  A.dt_min = reinterpret_cast<unsigned long long*>(ctl + 1);
  A.status = reinterpret_cast<int*>(ctl + 2);
  A.gamma = cfg->gamma;
  A.bc_p = cfg->bc_pressure;
  A.cfl = cfg->cfl;
  A.G = G;
  for (int k = 0; k < 4; ++k) {
    A.Pin[k] = prim[k];
    A.Uk[k] = prim[k];
    A.Uo[k] = res[k];
  }
  const int W = threads - 2 * ng;
  const int recon = recon_of_limiter(cfg->limiter);
  NA_CK(launch_stage<double>(cfg->flux, recon, dim3((ni + W - 1) / W, (nj + A.rows_per_cta - 1) /
                                                                          A.rows_per_cta),
                             threads, s, A, K));
  const int4 bc = make_int4(cfg->bc[0], cfg->bc[1], cfg->bc[2], cfg->bc[3]);
  const long long nh = hld * (nj + 2 * ng);
  int blocks = (int)((nh + 255) / 256);
  blocks = blocks > 4864 ? 4864 : blocks;
  // the BC-filled halo-padded primitives written back to the caller (flux_solver.f90:138-185);
  // no pressure-input edge states (that boundary is refused above)
  fill_ghosts_kernel<<<blocks, 256, 0, s>>>(ni, nj, pitch, ng, bc, cfg->gamma, cfg->bc_pressure,
                                            nullptr, prim[0], prim[1], prim[2], prim[3], gh[0],
                                            gh[1], gh[2], gh[3], hld);
  NA_CK(cudaGetLastError());
  for (int k = 0; k < 4; ++k)
    NA_CK(cudaMemcpy2DAsync(host_prim[k], (size_t)ld * sizeof(double), gh[k],
                            (size_t)hld * sizeof(double), (size_t)hld * sizeof(double),
                            (size_t)(nj + 2 * ng), cudaMemcpyDeviceToHost, s));
  for (int k = 0; k < 4; ++k) {
    for (int j = 0; j < nj + 2 * ng; ++j)
      std::memset(host_res[k] + (size_t)j * ld, 0, sizeof(double) * (size_t)hld);
    NA_CK(cudaMemcpy2DAsync(host_res[k] + (size_t)ng * ld + ng, (size_t)ld * sizeof(double),
                            res[k], (size_t)pitch * sizeof(double), (size_t)ni * sizeof(double),
                            (size_t)nj, cudaMemcpyDeviceToHost, s));
  }
  NA_CK(cudaStreamSynchronize(s));
#undef NA_CK
  return CATO_OK;
}
