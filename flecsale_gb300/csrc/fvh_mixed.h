// Mixed-precision form of the hydro step: FP32 reconstruction and Riemann
// fluxes; FP64 cell state, conservative update and dt reduction.
#pragma once

#include <cuda_runtime.h>

#include "flecsale_gb300.h"

namespace fvh {
namespace mixed {

struct workspace;

fvh_status create(const fvh_mesh_view &m, const fvh_params &p, workspace **out);
void destroy(workspace *w);

// Called after each kernel launch of a step when profiling (name is static).
struct launch_mark {
  void (*fn)(void *ctx, const char *name) = nullptr;
  void *ctx = nullptr;
  void operator()(const char *name) const {
    if (fn) fn(ctx, name);
  }
};

// One full time step (dt + two half-dt stages) on the FP64 state.
cudaError_t step(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                 const fvh_state_view &s, double *soln_time, double *dt,
                 double *partial, int dt_blocks, fvh_device_status *status,
                 cudaStream_t st, const launch_mark &mark = launch_mark());

// Kernel launches per step.
int launches_per_step(const fvh_params &p);

}  // namespace mixed
}  // namespace fvh
