// cato_batch.cuh -- many independent grid instances of uneven sizes advanced together: one
// persistent launch per RK stage (and per flux/reconstruction group) walks a work list of
// (instance, tile) items through a device-side queue, so 256 grids cost the launches of one.
// Every instance keeps its own dt, time, iteration and stop condition in a device descriptor,
// so a chunk of steps needs no host round trip and can be captured in a CUDA graph.
#pragma once

#include "cato_ctl.cuh"
#include "cato_stage.cuh"

namespace cato {

struct InstDesc {
  StepCtl ctl;             // per-instance step control (dt, time, iteration, stop, status)
  int ni, nj, pitch, ng;
  int bc[4];
  int limiter, rows_per_cta, flux, recon;
  int raw_pending;         // the first stage uses the uploaded primitives as is
  int prec;                // 0 FP64, 1 mixed, 2 mixed_df (one FP64 layout for all)
  int in_use;
  double gamma, cfl, bc_p;
  Geom G;
  FluxConsts<double> K64;
  FluxConsts<float> K32;
  FluxConsts<df> Kdf;
  double* U[4];            // U^n
  double* S[2][4];         // stage buffers
  double* prim_raw[4];
};

struct BatchStageArgs {
  InstDesc* descs;
  const int4* items;       // (instance, tile x, tile y, rows per tile)
  int n_items;
  int* counter;            // work-queue head, zeroed by batch_step_begin
  int stage, kind, last;
  double a, b, coef;
};

// Build one instance's StageArgs for this stage: the device-side twin of the single-instance
// host sequencing (cato_capi.cu enqueue_step).
template <typename R>
__device__ __forceinline__ void batch_stage_args(InstDesc* d, const BatchStageArgs& B,
                                                 StageArgs& A) {
  A.ni = d->ni;
  A.nj = d->nj;
  A.pitch = d->pitch;
#pragma unroll
  for (int k = 0; k < 4; ++k) A.bc[k] = d->bc[k];
  A.limiter = d->limiter;
  A.rows_per_cta = d->rows_per_cta;
  A.kind = B.kind;
  A.last = B.last;
  A.a = B.a;
  A.b = B.b;
  A.coef = B.coef;
  A.dt = &d->ctl.dt;
  A.active = nullptr;
  A.dt_min = &d->ctl.dt_min;
  A.status = &d->ctl.status;
  A.gamma = d->gamma;
  A.bc_p = d->bc_p;
  A.cfl = d->cfl;
  A.G = d->G;
  // single-handle features the batch does not carry (configurations are rejected at add)
  A.pbc_edge = nullptr;
  A.pbc_ng = 0;
  A.src_q = nullptr;
  const bool raw = (B.stage == 0) && d->raw_pending;
  double* const* prev = (B.stage == 0) ? d->U : d->S[(B.stage - 1) & 1];
  double* const* out = B.last ? d->U : d->S[B.stage & 1];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    A.Uk[v] = prev[v];
    A.Ua[v] = d->U[v];
    A.Uo[v] = out[v];
    A.Pin[v] = raw ? d->prim_raw[v] : nullptr;
  }
}

template <typename R, int NG, int FLUX, int RECON>
__global__ void __launch_bounds__(256, batch_min_blocks<R, FLUX>())
    batch_stage_kernel(const BatchStageArgs B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  for (;;) {
    __syncthreads();  // the previous tile is done with shared memory and s_item
    if (threadIdx.x == 0) s_item = atomicAdd(B.counter, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= B.n_items) break;
    const int4 w = B.items[it];
    InstDesc* d = B.descs + w.x;
    if (!d->ctl.active) continue;
    StageArgs A;
    batch_stage_args<R>(d, B, A);
    A.rows_per_cta = w.w;
    if constexpr (Prec<R>::kind == 0)
      stage_tile<R, NG, FLUX, RECON, true>(A, d->K64, w.y, w.z, smem_raw);
    else if constexpr (Prec<R>::kind == 1)
      // no rectilinear grid, source or pressure input in a batch: the lean FP32 kernel
      stage_tile<R, NG, FLUX, RECON, false>(A, d->K32, w.y, w.z, smem_raw);
    else
      stage_tile<R, NG, FLUX, RECON, true>(A, d->Kdf, w.y, w.z, smem_raw);
  }
}

}  // namespace cato
