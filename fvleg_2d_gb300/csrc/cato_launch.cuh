// cato_launch.cuh -- host-side launchers of the stage kernel, instantiated per (precision, flux)
// in separate translation units (stage_inst.cu compiled once per pair) so that the FP64 ones can
// be built with --fmad=false and the build parallelises.
#pragma once

#include <atomic>

#include "cato_batch.cuh"
#include "cato_stage.cuh"

namespace cato {

// A kernel's function attributes (here its dynamic shared-memory limit) belong to the GPU that
// is current when they are set, so the "already set" flags are kept per device.
constexpr int kMaxDevices = 64;
struct PerDevice {
  std::atomic<bool> done[kMaxDevices] = {};
  std::atomic<int> sms[kMaxDevices] = {};
};
// the current device, or -1 when it cannot be read or lies beyond kMaxDevices
inline int launch_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return -1;
  return dev;
}

template <typename R, int NG, int FLUX, int RECON, bool EXT, int MB = min_blocks<R>()>
cudaError_t launch_stage_ext(dim3 grid, int threads, cudaStream_t stream, const StageArgs& A,
                             const FluxConsts<R>& K) {
  static PerDevice attr;
  const size_t smem = stage_smem_bytes<R>(threads, NG);
  const int dev = launch_device();
  if (dev < 0) return cudaErrorInvalidDevice;
  if (!attr.done[dev].load(std::memory_order_acquire)) {
    cudaError_t e = cudaFuncSetAttribute(stage_kernel<R, NG, FLUX, RECON, EXT, MB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)stage_smem_bytes<R>(256, 3));
    if (e != cudaSuccess) return e;
    attr.done[dev].store(true, std::memory_order_release);
  }
  if (grid.x == 0 || grid.y == 0) return cudaSuccess;  // attribute warm-up only
  stage_kernel<R, NG, FLUX, RECON, EXT, MB><<<grid, threads, smem, stream>>>(A, K);
  return cudaGetLastError();
}

// The FP32 path has a lean variant without the rectilinear, source and pressure-input code
// (it is issue-bound: those checks cost ~3 %); double-float keeps one kernel.  The FP64 path
// has one kernel per register budget (variant 0: the compiler's choice, 1: at most 128, 2: at
// most 85).
template <typename R, int NG, int FLUX, int RECON>
cudaError_t launch_stage_one(dim3 grid, int threads, cudaStream_t stream, const StageArgs& A,
                             const FluxConsts<R>& K, int variant) {
  const bool warm = grid.x == 0 || grid.y == 0;  // attribute warm-up of every variant
  if constexpr (Prec<R>::kind == 1) {
    if (warm) {
      cudaError_t e = launch_stage_ext<R, NG, FLUX, RECON, false>(grid, threads, stream, A, K);
      if (e != cudaSuccess) return e;
      return launch_stage_ext<R, NG, FLUX, RECON, true>(grid, threads, stream, A, K);
    }
    if (!stage_needs_ext(A))
      return launch_stage_ext<R, NG, FLUX, RECON, false>(grid, threads, stream, A, K);
  }
  if constexpr (Prec<R>::kind == 0) {
    if (warm) {
      cudaError_t e = launch_stage_ext<R, NG, FLUX, RECON, true, CATO_F64_MIN_BLOCKS_ALT>(
          grid, threads, stream, A, K);
      if (e != cudaSuccess) return e;
      e = launch_stage_ext<R, NG, FLUX, RECON, true, CATO_F64_MIN_BLOCKS_ALT2>(grid, threads,
                                                                              stream, A, K);
      if (e != cudaSuccess) return e;
    } else if (variant == 1) {
      return launch_stage_ext<R, NG, FLUX, RECON, true, CATO_F64_MIN_BLOCKS_ALT>(grid, threads,
                                                                                stream, A, K);
    } else if (variant == 2) {
      return launch_stage_ext<R, NG, FLUX, RECON, true, CATO_F64_MIN_BLOCKS_ALT2>(grid, threads,
                                                                                 stream, A, K);
    }
  }
  return launch_stage_ext<R, NG, FLUX, RECON, true>(grid, threads, stream, A, K);
}

// recon: 0 = TVD2 (minmod / superbee / van Leer), 3 = MLP3, 5 = MLP5
template <typename R, int FLUX>
inline cudaError_t launch_stage_flux(int recon, dim3 grid, int threads, cudaStream_t stream,
                                     const StageArgs& A, const FluxConsts<R>& K, int variant) {
  switch (recon) {
    case 0: return launch_stage_one<R, 2, FLUX, 0>(grid, threads, stream, A, K, variant);
    case 3: return launch_stage_one<R, 2, FLUX, 3>(grid, threads, stream, A, K, variant);
    case 5: return launch_stage_one<R, 3, FLUX, 5>(grid, threads, stream, A, K, variant);
    default: return cudaErrorInvalidValue;
  }
}

// Persistent batch launch: as many CTAs as can be resident, each looping over work items.
template <typename R, int NG, int FLUX, int RECON>
cudaError_t launch_batch_one(int threads, cudaStream_t stream, const BatchStageArgs& B) {
  static PerDevice attr;
  const size_t smem = stage_smem_bytes<R>(threads, NG);
  const int dev = launch_device();
  if (dev < 0) return cudaErrorInvalidDevice;
  if (!attr.done[dev].load(std::memory_order_acquire)) {
    cudaError_t e = cudaFuncSetAttribute(batch_stage_kernel<R, NG, FLUX, RECON>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)stage_smem_bytes<R>(256, 3));
    if (e != cudaSuccess) return e;
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    attr.sms[dev].store(n > 0 ? n : 1);
    attr.done[dev].store(true, std::memory_order_release);
  }
  if (B.n_items <= 0) return cudaSuccess;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, batch_stage_kernel<R, NG, FLUX, RECON>, threads, smem);
  if (e != cudaSuccess) return e;
  long long grid = (long long)(per_sm > 0 ? per_sm : 1) * attr.sms[dev].load();
  if (grid > B.n_items) grid = B.n_items;
  batch_stage_kernel<R, NG, FLUX, RECON><<<(unsigned)grid, threads, smem, stream>>>(B);
  return cudaGetLastError();
}

template <typename R, int FLUX>
inline cudaError_t launch_batch_flux(int recon, int threads, cudaStream_t stream,
                                     const BatchStageArgs& B) {
  switch (recon) {
    case 0: return launch_batch_one<R, 2, FLUX, 0>(threads, stream, B);
    case 3: return launch_batch_one<R, 2, FLUX, 3>(threads, stream, B);
    case 5: return launch_batch_one<R, 3, FLUX, 5>(threads, stream, B);
    default: return cudaErrorInvalidValue;
  }
}

// Every (precision, NG, flux, reconstruction) kernel is instantiated in exactly one translation
// unit (stage_inst.cu, compiled once per precision and flux, and for the slow double-float units
// once per reconstruction and kernel kind); everywhere else these are extern.
#define CATO_DECLARE_ONE(R, F, NG, RC)                                                         \
  extern template cudaError_t launch_stage_one<R, NG, F, RC>(dim3, int, cudaStream_t,          \
                                                             const StageArgs&,                 \
                                                             const FluxConsts<R>&, int);       \
  extern template cudaError_t launch_batch_one<R, NG, F, RC>(int, cudaStream_t,               \
                                                             const BatchStageArgs&);
#define CATO_DECLARE_STAGE(R, F) \
  CATO_DECLARE_ONE(R, F, 2, 0) CATO_DECLARE_ONE(R, F, 2, 3) CATO_DECLARE_ONE(R, F, 3, 5)
#define CATO_DECLARE_PREC(R)                                                      \
  CATO_DECLARE_STAGE(R, 0) CATO_DECLARE_STAGE(R, 1) CATO_DECLARE_STAGE(R, 2)      \
  CATO_DECLARE_STAGE(R, 3) CATO_DECLARE_STAGE(R, 4) CATO_DECLARE_STAGE(R, 5)      \
  CATO_DECLARE_STAGE(R, 6) CATO_DECLARE_STAGE(R, 7) CATO_DECLARE_STAGE(R, 8)
CATO_DECLARE_PREC(double)
CATO_DECLARE_PREC(float)
CATO_DECLARE_PREC(df)
#undef CATO_DECLARE_PREC
#undef CATO_DECLARE_STAGE
#undef CATO_DECLARE_ONE

// variant: the FP64 kernel's register budget (0, 1 or 2, see launch_stage_one); ignored otherwise
template <typename R>
inline cudaError_t launch_stage(int flux, int recon, dim3 grid, int threads, cudaStream_t s,
                                const StageArgs& A, const FluxConsts<R>& K, int variant = 0) {
  switch (flux) {
    case 0: return launch_stage_flux<R, 0>(recon, grid, threads, s, A, K, variant);
    case 1: return launch_stage_flux<R, 1>(recon, grid, threads, s, A, K, variant);
    case 2: return launch_stage_flux<R, 2>(recon, grid, threads, s, A, K, variant);
    case 3: return launch_stage_flux<R, 3>(recon, grid, threads, s, A, K, variant);
    case 4: return launch_stage_flux<R, 4>(recon, grid, threads, s, A, K, variant);
    case 5: return launch_stage_flux<R, 5>(recon, grid, threads, s, A, K, variant);
    case 6: return launch_stage_flux<R, 6>(recon, grid, threads, s, A, K, variant);
    case 7: return launch_stage_flux<R, 7>(recon, grid, threads, s, A, K, variant);
    case 8: return launch_stage_flux<R, 8>(recon, grid, threads, s, A, K, variant);
    default: return cudaErrorInvalidValue;
  }
}

template <typename R>
inline cudaError_t launch_batch(int flux, int recon, int threads, cudaStream_t s,
                                const BatchStageArgs& B) {
  switch (flux) {
    case 0: return launch_batch_flux<R, 0>(recon, threads, s, B);
    case 1: return launch_batch_flux<R, 1>(recon, threads, s, B);
    case 2: return launch_batch_flux<R, 2>(recon, threads, s, B);
    case 3: return launch_batch_flux<R, 3>(recon, threads, s, B);
    case 4: return launch_batch_flux<R, 4>(recon, threads, s, B);
    case 5: return launch_batch_flux<R, 5>(recon, threads, s, B);
    case 6: return launch_batch_flux<R, 6>(recon, threads, s, B);
    case 7: return launch_batch_flux<R, 7>(recon, threads, s, B);
    case 8: return launch_batch_flux<R, 8>(recon, threads, s, B);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cato
