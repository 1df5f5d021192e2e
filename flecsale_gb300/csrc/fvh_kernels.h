// Kernel launch configuration and device helpers shared by the kernel files.
#pragma once

#include <cuda_runtime.h>

#include "flecsale_gb300.h"

namespace fvh {

constexpr int kDtThreads = 256;
constexpr int kCellThreads = 128;
constexpr int kFaceThreads = 128;
// Upper bound on the blocks of the dt partial-max pass: 152 SMs x 8.
constexpr int kDtMaxBlocks = 1216;

// Key for the device status word: the smallest (cell, code) wins an atomicMin.
__host__ __device__ inline unsigned long long status_key(long long cell, int code) {
  return ((unsigned long long)cell << 8) | (unsigned long long)(code & 0xff);
}

#ifdef __CUDACC__
// Block-wide maximum with the reference's std::max semantics; all threads of
// the block must call it; the result is valid in thread 0.
__device__ inline double block_max(double v) {
  __shared__ double warp_max[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (v < w) ? w : v;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warp_max[warp] = v;
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? warp_max[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double w = __shfl_xor_sync(0xffffffffu, v, o);
      v = (v < w) ? w : v;
    }
  }
  return v;
}
#endif

namespace plain {
// slot_dx / lsq: optional per-mesh tables (null = compute on the fly; the
// results are the same either way)
template <int D>
cudaError_t launch_dt(const fvh_mesh_view &m, const fvh_state_view &s,
                      const fvh_params &p, const double *soln_time, double *dt,
                      double *partial, int nblocks, fvh_device_status *status,
                      cudaStream_t st, const double *slot_dx = nullptr);
template <int D>
cudaError_t launch_gradients(const fvh_mesh_view &m, const fvh_state_view &s,
                             const fvh_gradient_view &g, const fvh_params &p,
                             cudaStream_t st, const double *lsq = nullptr);
template <int D>
cudaError_t build_tables(const fvh_mesh_view &m, double *lsq, double *slot_dx);
int lsq_doubles_per_cell(int dim);
template <int D>
cudaError_t launch_fluxes(const fvh_mesh_view &m, const fvh_state_view &s,
                          const fvh_gradient_view &g, const fvh_flux_view &fl,
                          const fvh_params &p, cudaStream_t st);
template <int D>
cudaError_t launch_update(const fvh_mesh_view &m, const fvh_params &p, const double *dt,
                          double factor, const fvh_flux_view &fl,
                          const fvh_state_view &s, double *soln_time,
                          fvh_device_status *status, cudaStream_t st);
}  // namespace plain

}  // namespace fvh
