// Instantiations of the stage kernel family.  The build compiles this file once per
// (precision, flux) pair with -DCATO_REAL=double|float|df -DCATO_FLUX=<0..8>, and the slow
// double-float pairs once more per reconstruction and kernel kind (-DCATO_RECON=0|3|5,
// -DCATO_PART=1 single-grid stage kernels | 2 persistent batch kernels), so that the build
// parallelises.  The FP64 objects are built with --fmad=false so that every reference operation
// rounds on its own.
#include "cato_launch.cuh"

#ifndef CATO_REAL
#error "CATO_REAL must be defined (double, float or df)"
#endif
#ifndef CATO_FLUX
#error "CATO_FLUX must be defined (0..8)"
#endif
#ifndef CATO_PART
#define CATO_PART 0  // both kinds
#endif

#define CATO_INST_STAGE(NG, RC)                                                               \
  template cudaError_t launch_stage_one<CATO_REAL, NG, CATO_FLUX, RC>(                        \
      dim3, int, cudaStream_t, const StageArgs&, const FluxConsts<CATO_REAL>&, int);
#define CATO_INST_BATCH(NG, RC)                                                               \
  template cudaError_t launch_batch_one<CATO_REAL, NG, CATO_FLUX, RC>(int, cudaStream_t,      \
                                                                      const BatchStageArgs&);
#if CATO_PART == 0
#define CATO_INST(NG, RC) CATO_INST_STAGE(NG, RC) CATO_INST_BATCH(NG, RC)
#elif CATO_PART == 1
#define CATO_INST(NG, RC) CATO_INST_STAGE(NG, RC)
#else
#define CATO_INST(NG, RC) CATO_INST_BATCH(NG, RC)
#endif

namespace cato {
#if !defined(CATO_RECON) || CATO_RECON == 0
CATO_INST(2, 0)
#endif
#if !defined(CATO_RECON) || CATO_RECON == 3
CATO_INST(2, 3)
#endif
#if !defined(CATO_RECON) || CATO_RECON == 5
CATO_INST(3, 5)
#endif
}  // namespace cato
