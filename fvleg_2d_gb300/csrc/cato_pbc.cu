// Launchers of the +x pressure-input boundary kernels for the three compute types.  Built with
// --fmad=false like the FP64 stage kernels, so that the FP64 primitives and the boundary state
// round exactly as the reference's operations do.
#include "cato_pbc.cuh"

namespace cato {

template <typename R>
static cudaError_t launch_pbc_t(const StageArgs& A, const PbcArgs& P, cudaStream_t s) {
  pbc_max_kernel<R><<<1, 1024, 0, s>>>(A, P);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int rows = A.nj + 2 * P.ng;
  pbc_edge_kernel<R><<<(rows + 63) / 64, 64, 0, s>>>(A, P);
  return cudaGetLastError();
}

cudaError_t launch_pbc(int precision, const StageArgs& A, const PbcArgs& P, cudaStream_t s) {
  switch (precision) {
    case 0: return launch_pbc_t<double>(A, P, s);
    case 1: return launch_pbc_t<float>(A, P, s);
    case 2: return launch_pbc_t<df>(A, P, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cato
