// Argument checks and CUDA error mapping shared by the C entry points (CUDA
// translation units only).
#pragma once

#include <cuda_runtime.h>

#include "flecsale_gb300.h"

namespace fvh {

inline fvh_status from_cuda(cudaError_t e) {
  if (e == cudaSuccess) return FVH_OK;
  if (e == cudaErrorMemoryAllocation) return FVH_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return FVH_ERR_NO_DEVICE;
  return FVH_ERR_CUDA;
}

inline bool mesh_ok(const fvh_mesh_view *m) {
  if (!m || (m->dim != 2 && m->dim != 3) || m->num_cells <= 0 || m->num_faces <= 0)
    return false;
  if (!m->face_cells || !m->cell_face_offsets || !m->cell_faces || !m->cell_nbr_offsets ||
      !m->cell_nbrs || !m->cell_vertex_offsets || !m->cell_vertices || !m->cell_volume ||
      !m->face_area)
    return false;
  for (int d = 0; d < m->dim; ++d)
    if (!m->cell_centroid[d] || !m->face_centroid[d] || !m->face_normal[d] ||
        !m->vertex_coord[d])
      return false;
  return true;
}

inline bool state_ok(const fvh_state_view *s, int dim) {
  if (!s || !s->density || !s->internal_energy || !s->pressure || !s->temperature ||
      !s->sound_speed)
    return false;
  for (int d = 0; d < dim; ++d)
    if (!s->velocity[d]) return false;
  return true;
}

inline bool grads_ok(const fvh_gradient_view *g, int dim) {
  if (!g) return false;
  for (int i = 0; i < dim; ++i) {
    if (!g->density[i] || !g->internal_energy[i] || !g->pressure[i] || !g->sound_speed[i])
      return false;
    for (int d = 0; d < dim; ++d)
      if (!g->velocity[d][i]) return false;
  }
  return true;
}

inline bool flux_ok(const fvh_flux_view *f, int dim) {
  if (!f || !f->mass || !f->energy) return false;
  for (int d = 0; d < dim; ++d)
    if (!f->momentum[d]) return false;
  return true;
}

inline bool params_ok(const fvh_params *p, int dim) {
  return p && p->dim == dim && p->flux_kind >= 0 && p->flux_kind <= 2 &&
         p->limiter >= 0 && p->limiter <= 1 && (p->order == 1 || p->order == 2) &&
         (p->precision == FVH_PRECISION_FP64 || p->precision == FVH_PRECISION_MIXED) &&
         (p->boundary == FVH_BOUNDARY_WALL || p->boundary == FVH_BOUNDARY_OUTFLOW) &&
         p->gamma > 1 && p->cv > 0 && p->cfl > 0;
}

}  // namespace fvh
