// cato_ctl.cuh -- device-resident step control shared by the single-instance and batch paths.
#pragma once

#include <cuda_runtime.h>

namespace cato {

// Device-resident step control: lets a chunk of steps run (and be captured in a CUDA graph)
// without host round trips.  `active` gates every kernel of a step.
struct StepCtl {
  double dt;          // dt of the current step
  double time;        // simulation time after the last active step
  double t_end;       // stop once time >= t_end (main.f90:138)
  double fixed_dt;    // > 0: use this dt instead of the CFL dt (use_constant_delta_t)
  long long iter;     // iteration counter
  long long max_iter; // stop once iter >= max_iter
  unsigned long long dt_min;  // CFL dt of the current state (bits; ~0 = none)
  int active;
  int status;         // ST_* bits of the current state
  double t_create;    // time the state was created at (upload / set_time): the flux solver of
                      // the persistent fluid keeps it under rk(m,n) (pressure-input table time)
  double t_step;      // time at the start of the current step (energy source term time)
};

__device__ __forceinline__ double decode_dt(unsigned long long b) {
  return b == ~0ULL ? INFINITY : __longlong_as_double((long long)b);
}

}  // namespace cato
