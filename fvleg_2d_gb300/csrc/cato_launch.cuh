// cato_launch.cuh -- host-side launchers of the stage kernel, instantiated per (precision, flux)
// in separate translation units (stage_inst.cu compiled once per pair) so that the FP64 ones can
// be built with --fmad=false and the build parallelises.
#pragma once

#include <atomic>

#include "cato_stage.cuh"

namespace cato {

// recon: 0 = TVD2 (minmod / superbee / van Leer), 3 = MLP3, 5 = MLP5
template <typename R, int FLUX>
cudaError_t launch_stage_flux(int recon, dim3 grid, int threads, cudaStream_t stream,
                              const StageArgs& A, const FluxConsts<R>& K);

template <typename R, int NG, int FLUX, int RECON>
cudaError_t launch_stage_one(dim3 grid, int threads, cudaStream_t stream, const StageArgs& A,
                             const FluxConsts<R>& K) {
  static std::atomic<bool> attr_done{false};
  const size_t smem = stage_smem_bytes<R>(threads, NG);
  if (!attr_done.load(std::memory_order_acquire)) {
    cudaError_t e = cudaFuncSetAttribute(stage_kernel<R, NG, FLUX, RECON>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)stage_smem_bytes<R>(256, 3));
    if (e != cudaSuccess) return e;
    attr_done.store(true, std::memory_order_release);
  }
  if (grid.x == 0 || grid.y == 0) return cudaSuccess;  // attribute warm-up only
  stage_kernel<R, NG, FLUX, RECON><<<grid, threads, smem, stream>>>(A, K);
  return cudaGetLastError();
}

template <typename R, int FLUX>
cudaError_t launch_stage_flux(int recon, dim3 grid, int threads, cudaStream_t stream,
                              const StageArgs& A, const FluxConsts<R>& K) {
  switch (recon) {
    case 0: return launch_stage_one<R, 2, FLUX, 0>(grid, threads, stream, A, K);
    case 3: return launch_stage_one<R, 2, FLUX, 3>(grid, threads, stream, A, K);
    case 5: return launch_stage_one<R, 3, FLUX, 5>(grid, threads, stream, A, K);
    default: return cudaErrorInvalidValue;
  }
}

#define CATO_DECLARE_STAGE(R, F)                                                             \
  extern template cudaError_t launch_stage_flux<R, F>(int, dim3, int, cudaStream_t,         \
                                                      const StageArgs&, const FluxConsts<R>&);
CATO_DECLARE_STAGE(double, 0) CATO_DECLARE_STAGE(double, 1) CATO_DECLARE_STAGE(double, 2)
CATO_DECLARE_STAGE(double, 3) CATO_DECLARE_STAGE(double, 4) CATO_DECLARE_STAGE(double, 5)
CATO_DECLARE_STAGE(double, 6) CATO_DECLARE_STAGE(double, 7)
CATO_DECLARE_STAGE(float, 0) CATO_DECLARE_STAGE(float, 1) CATO_DECLARE_STAGE(float, 2)
CATO_DECLARE_STAGE(float, 3) CATO_DECLARE_STAGE(float, 4) CATO_DECLARE_STAGE(float, 5)
CATO_DECLARE_STAGE(float, 6) CATO_DECLARE_STAGE(float, 7)
#undef CATO_DECLARE_STAGE

template <typename R>
inline cudaError_t launch_stage(int flux, int recon, dim3 grid, int threads, cudaStream_t s,
                                const StageArgs& A, const FluxConsts<R>& K) {
  switch (flux) {
    case 0: return launch_stage_flux<R, 0>(recon, grid, threads, s, A, K);
    case 1: return launch_stage_flux<R, 1>(recon, grid, threads, s, A, K);
    case 2: return launch_stage_flux<R, 2>(recon, grid, threads, s, A, K);
    case 3: return launch_stage_flux<R, 3>(recon, grid, threads, s, A, K);
    case 4: return launch_stage_flux<R, 4>(recon, grid, threads, s, A, K);
    case 5: return launch_stage_flux<R, 5>(recon, grid, threads, s, A, K);
    case 6: return launch_stage_flux<R, 6>(recon, grid, threads, s, A, K);
    case 7: return launch_stage_flux<R, 7>(recon, grid, threads, s, A, K);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cato
