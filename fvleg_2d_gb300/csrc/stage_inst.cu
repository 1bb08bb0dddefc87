// One (precision, flux) instantiation of the stage kernel family.  The build compiles this file
// once per pair with -DCATO_REAL=double|float|df -DCATO_FLUX=<0..7>; the FP64 objects are built
// with --fmad=false so that every reference operation rounds on its own.
#include "cato_launch.cuh"

#ifndef CATO_REAL
#error "CATO_REAL must be defined (double, float or df)"
#endif
#ifndef CATO_FLUX
#error "CATO_FLUX must be defined (0..7)"
#endif

namespace cato {
template cudaError_t launch_stage_flux<CATO_REAL, CATO_FLUX>(int, dim3, int, cudaStream_t,
                                                             const StageArgs&,
                                                             const FluxConsts<CATO_REAL>&);
template cudaError_t launch_batch_flux<CATO_REAL, CATO_FLUX>(int, int, cudaStream_t,
                                                             const BatchStageArgs&);
}  // namespace cato
