// fvh_evaluate_time_step_noalloc: the CFL time-step reduction for callers that
// cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: a task runtime that owns all device
// memory through its own pool and hands a task only the field buffers it
// manages, or a hot loop that must not pay cudaMalloc's implicit device
// synchronisation.  They still pass the inputs (mesh, state, solution time)
// and the outputs (dt, status word); the per-block partial maxima that
// fvh_evaluate_time_step keeps in a caller-supplied workspace live here in a
// fixed device array inside the library instead.
//
// The array holds kMaxBlocks doubles (64 KiB).  It is a module global, so every
// GPU that loads the library keeps it until the process exits.  One block of
// kDtThreads threads covers kDtThreads cells, so the largest mesh accepted is
// kMaxBlocks * kDtThreads = 2,097,152 cells; larger meshes are rejected with
// FVH_ERR_CAPACITY before anything is launched.
//
// All calls share the one array.  Each call writes every partial it later reads
// before reading it, so nothing has to be cleared between calls, but two calls
// whose kernels overlap on the GPU (for example on two streams) race on it.
//
// The arguments are checked exactly as fvh_evaluate_time_step checks them, and
// CUDA errors map to the same status codes.  The kernels are the same; only
// the number of blocks differs above kDtMaxBlocks blocks (fvh_evaluate_time_step
// then strides each block over more cells), and the largest of the per-block
// maxima does not depend on how the cells were split, so both entry points
// give the same dt for every state without a NaN.
#include <cuda_runtime.h>

#include <atomic>

#include "flecsale_gb300.h"
#include "fvh_checks.h"
#include "fvh_kernels.h"

namespace {

constexpr int kMaxBlocks = 8192;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_dt_partials[kMaxBlocks];

// Device address of g_dt_partials, per device.  In host code the name
// g_dt_partials is only a host-side stand-in, so the address must come from
// cudaGetSymbolAddress with the device current.
std::atomic<double *> g_partials_addr[kMaxDevices];

fvh_status partials_for_current_device(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FVH_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return FVH_ERR_UNSUPPORTED;
  double *p = g_partials_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    const cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_dt_partials);
    if (e != cudaSuccess) return fvh::from_cuda(e);
    if (!p) return FVH_ERR_CUDA;
    g_partials_addr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return FVH_OK;
}

}  // namespace

extern "C" {

int32_t fvh_time_step_noalloc_max_cells(void) { return kMaxBlocks * fvh::kDtThreads; }

fvh_status fvh_evaluate_time_step_noalloc(const fvh_mesh_view *mesh,
                                          const fvh_state_view *state,
                                          const fvh_params *params,
                                          const double *d_soln_time, double *d_dt,
                                          fvh_device_status *d_status,
                                          fvh_stream_t stream) {
  if (!fvh::mesh_ok(mesh) || !fvh::state_ok(state, mesh->dim) ||
      !fvh::params_ok(params, mesh->dim) || !d_soln_time || !d_dt || !d_status)
    return FVH_ERR_INVALID_ARGUMENT;
  const long long nblocks =
      ((long long)mesh->num_cells + fvh::kDtThreads - 1) / fvh::kDtThreads;
  if (nblocks > kMaxBlocks) return FVH_ERR_CAPACITY;
  double *partial = nullptr;
  const fvh_status st = partials_for_current_device(&partial);
  if (st != FVH_OK) return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const cudaError_t e =
      mesh->dim == 2
          ? fvh::plain::launch_dt<2>(*mesh, *state, *params, d_soln_time, d_dt, partial,
                                     (int)nblocks, d_status, s)
          : fvh::plain::launch_dt<3>(*mesh, *state, *params, d_soln_time, d_dt, partial,
                                     (int)nblocks, d_status, s);
  return fvh::from_cuda(e);
}

}  // extern "C"
