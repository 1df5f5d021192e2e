// Kernel launch configuration and device helpers shared by the kernel files.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

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
// Geometry-only tables of the FP64 solver, built once per mesh with the same
// operations the kernels would perform on the fly, so the results are the same
// either way (a null member is computed on the fly).
struct tables {
  const double *lsq = nullptr;      // per cell: least-squares matrix terms, SoA planes
  const double *slot_dx = nullptr;  // per (cell, face) slot: V_c / A_f
  const double *nbr_dx = nullptr;   // per (cell, neighbour) slot: x_nbr - x_c, D doubles
  const double *vtx_dx = nullptr;   // per (cell, vertex) slot: x_v - x_c, D doubles
  const double *face_dx = nullptr;  // per face: x_f - x_c0 then x_f - x_c1, 2D doubles
};
// doubles the tables of a mesh take (nnz_*: the CSR list lengths)
size_t table_doubles(int dim, int64_t nc, int64_t nf, int64_t nnz_cf, int64_t nnz_nb,
                     int64_t nnz_cv);
// carves the tables out of `base` (table_doubles long) and fills them
template <int D>
cudaError_t build_tables(const fvh_mesh_view &m, double *base, int64_t nnz_cf,
                         int64_t nnz_nb, int64_t nnz_cv, tables *t);

template <int D>
cudaError_t launch_dt(const fvh_mesh_view &m, const fvh_state_view &s,
                      const fvh_params &p, const double *soln_time, double *dt,
                      double *partial, int nblocks, fvh_device_status *status,
                      cudaStream_t st, const double *slot_dx = nullptr,
                      const fvh_state_view *src = nullptr);
template <int D>
cudaError_t launch_gradients(const fvh_mesh_view &m, const fvh_state_view &s,
                             const fvh_gradient_view &g, const fvh_params &p,
                             cudaStream_t st, const tables &t = tables());
template <int D>
cudaError_t launch_fluxes(const fvh_mesh_view &m, const fvh_state_view &s,
                          const fvh_gradient_view &g, const fvh_flux_view &fl,
                          const fvh_params &p, cudaStream_t st, const tables &t = tables());
// Diagnostic: out[i] = a[i] op b[i] for op 0 mul, 1 add, 2 sub, 3 div on the
// integer pipes (fvh_sf64.cuh), 4..7 the same with the FP64 instructions,
// 8 / 9 the optimistic mul / div with their FP64 redo.
cudaError_t debug_sf64(int op, const double *a, const double *b, int64_t n, double *out,
                       cudaStream_t st);
// out (optional): a second copy of the new state, e.g. host-mapped planes of
// a caller that holds its state in host memory
template <int D>
cudaError_t launch_update(const fvh_mesh_view &m, const fvh_params &p, const double *dt,
                          double factor, const fvh_flux_view &fl,
                          const fvh_state_view &s, double *soln_time,
                          fvh_device_status *status, cudaStream_t st,
                          const fvh_state_view *out = nullptr);
}  // namespace plain

}  // namespace fvh
