// Mixed-precision form of the hydro step (sm_103a).
//
// Reconstruction, limiter and Riemann fluxes run in FP32; the cell state, the
// face-to-cell accumulation, the conservative update and the dt reduction stay
// in FP64.  Per time step (the structure of apps/hydro/driver.h:325-375):
//
//   pack_dt      FP64 state -> FP32 recon pack (AoS, 32 B/cell) and the
//                per-block max of (a+|v.n|) A/V for the CFL step (tasks.h:331-376)
//   dt_final     one block: dt = min(CFL/max, t_f - t) in FP64
//   gradients    FP32 vertex-neighbour least squares + Barth-Jespersen limiter
//                (tasks.h:145-321), FP32 AoS gradients
//   flux_update  cell-centric: for each face of the cell, reconstruct both
//                sides at the face centroid, Riemann/wall flux in FP32
//                (tasks.h:385-464), accumulate -/+F in FP64 in the cell's face
//                order, then the conservative FP64 update + EOS closure
//                (tasks.h:589-659); writes the FP64 state and, after the
//                predictor, the next FP32 pack
//   (gradients, flux_update again for the corrector)
//
// A face shared by two cells is evaluated by both with identical inputs and
// identical instructions, so both cells see the same bits: the update is
// conservative to FP64 rounding without a flux array in HBM and without atomics.
#include <cuda_runtime.h>

#include <cstdint>
#include <new>

#include "fvh_kernels.h"
#include "fvh_mixed.h"
#include "fvh_physics.cuh"

namespace fvh {
namespace mixed {

using phys::prim;
using phys::smax;
using phys::smin;

// per-cell AoS record sizes in float4 units
template <int D>
struct layout {
  static constexpr int NV = D + 4;             // d, v[D], e, p, a
  static constexpr int PACK4 = 2;              // d v.. p e a (8 floats)
  static constexpr int GRAD4 = D == 2 ? 3 : 6; // NV*D floats, padded
  static constexpr int CEN4 = D == 2 ? 1 : 2;  // centroid hi/lo
  static constexpr int FGEO4 = 1;              // normal[D], area
  static constexpr int FDX4 = D == 2 ? 1 : 2;  // x_f - x_c0, x_f - x_c1
};

struct workspace {
  int dim = 0, nc = 0, nf = 0, nv = 0;
  void *base = nullptr;
  float4 *pack = nullptr;    // FP32 recon pack of the predictor (from the FP64 state)
  float4 *pack2 = nullptr;   // pack of the corrector (written by the predictor update)
  float4 *grads = nullptr;
  float4 *ccen = nullptr;    // cell centroid hi/lo
  float4 *vcoord = nullptr;  // vertex coordinates hi/lo
  float4 *fgeo = nullptr;    // face normal + area
  float4 *fdx = nullptr;     // face centroid offsets from both cells
  double *inv_vol = nullptr; // 1/V (FP64)
};

// Load pack fields: slots (d, v0, v1, [v2,] p, e, a) in the AoS order
//   2D: f4[0] = (d, vx, vy, p)  f4[1] = (e, a, 0, 0)
//   3D: f4[0] = (d, vx, vy, vz) f4[1] = (p, e, a, 0)
template <int D>
__device__ __forceinline__ prim<float, D> load_pack(const float4 *pk, int c) {
  const float4 a = pk[2 * (size_t)c], b = pk[2 * (size_t)c + 1];
  prim<float, D> w;
  w.d = a.x;
  w.v[0] = a.y;
  w.v[1] = a.z;
  if (D == 2) {
    w.p = a.w;
    w.e = b.x;
    w.a = b.y;
  } else {
    w.v[D - 1] = a.w;
    w.p = b.x;
    w.e = b.y;
    w.a = b.z;
  }
  return w;
}

template <int D>
__device__ __forceinline__ void store_pack(float4 *pk, int c, float d, const float *v, float p,
                                           float e, float a) {
  if (D == 2) {
    pk[2 * (size_t)c] = make_float4(d, v[0], v[1], p);
    pk[2 * (size_t)c + 1] = make_float4(e, a, 0.f, 0.f);
  } else {
    pk[2 * (size_t)c] = make_float4(d, v[0], v[1], v[D - 1]);
    pk[2 * (size_t)c + 1] = make_float4(p, e, a, 0.f);
  }
}

// gradient record: g[k*D + i] = d u_k / d x_i, u = (d, v.., e, p, a)
template <int D>
__device__ __forceinline__ void load_grads(const float4 *gr, int c, float *g) {
  constexpr int G4 = layout<D>::GRAD4;
#pragma unroll
  for (int q = 0; q < G4; ++q) {
    const float4 t = gr[(size_t)G4 * c + q];
    g[4 * q] = t.x;
    g[4 * q + 1] = t.y;
    g[4 * q + 2] = t.z;
    g[4 * q + 3] = t.w;
  }
}

template <int D>
__device__ __forceinline__ void load_cen(const float4 *cc, int c, float *hi, float *lo) {
  if (D == 2) {
    const float4 t = cc[c];
    hi[0] = t.x; hi[1] = t.y; lo[0] = t.z; lo[1] = t.w;
  } else {
    const float4 a = cc[2 * (size_t)c], b = cc[2 * (size_t)c + 1];
    hi[0] = a.x; hi[1] = a.y; hi[D - 1] = a.z;
    lo[0] = b.x; lo[1] = b.y; lo[D - 1] = b.z;
  }
}

__device__ __forceinline__ float2 split(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

// ---------------------------------------------------------------------------
// setup: FP32 geometry derived once from the FP64 mesh
// ---------------------------------------------------------------------------
template <int D>
__global__ void setup_cells(const fvh_mesh_view m, workspace w) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.num_cells) return;
  float hi[3], lo[3];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    const float2 s = split(m.cell_centroid[i][c]);
    hi[i] = s.x;
    lo[i] = s.y;
  }
  if (D == 2) {
    w.ccen[c] = make_float4(hi[0], hi[1], lo[0], lo[1]);
  } else {
    w.ccen[2 * (size_t)c] = make_float4(hi[0], hi[1], hi[D - 1], 0.f);
    w.ccen[2 * (size_t)c + 1] = make_float4(lo[0], lo[1], lo[D - 1], 0.f);
  }
  w.inv_vol[c] = 1.0 / m.cell_volume[c];
}

template <int D>
__global__ void setup_vertices(const fvh_mesh_view m, workspace w) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.num_vertices) return;
  float hi[3], lo[3];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    const float2 s = split(m.vertex_coord[i][v]);
    hi[i] = s.x;
    lo[i] = s.y;
  }
  if (D == 2) {
    w.vcoord[v] = make_float4(hi[0], hi[1], lo[0], lo[1]);
  } else {
    w.vcoord[2 * (size_t)v] = make_float4(hi[0], hi[1], hi[D - 1], 0.f);
    w.vcoord[2 * (size_t)v + 1] = make_float4(lo[0], lo[1], lo[D - 1], 0.f);
  }
}

template <int D>
__global__ void setup_faces(const fvh_mesh_view m, workspace w) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.num_faces) return;
  const int c0 = m.face_cells[2 * (size_t)f], c1 = m.face_cells[2 * (size_t)f + 1];
  float n[3], d0[3], d1[3];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    n[i] = (float)m.face_normal[i][f];
    const double xf = m.face_centroid[i][f];
    d0[i] = (float)(xf - m.cell_centroid[i][c0]);
    d1[i] = c1 >= 0 ? (float)(xf - m.cell_centroid[i][c1]) : 0.f;
  }
  const float area = (float)m.face_area[f];
  if (D == 2) {
    w.fgeo[f] = make_float4(n[0], n[1], area, 0.f);
    w.fdx[f] = make_float4(d0[0], d0[1], d1[0], d1[1]);
  } else {
    w.fgeo[f] = make_float4(n[0], n[1], n[D - 1], area);
    w.fdx[2 * (size_t)f] = make_float4(d0[0], d0[1], d0[D - 1], 0.f);
    w.fdx[2 * (size_t)f + 1] = make_float4(d1[0], d1[1], d1[D - 1], 0.f);
  }
}

template <int D>
__device__ __forceinline__ void face_geo(const workspace &w, int f, float *n, float &area) {
  const float4 g = w.fgeo[f];
  n[0] = g.x;
  n[1] = g.y;
  if (D == 2) {
    area = g.z;
  } else {
    n[D - 1] = g.z;
    area = g.w;
  }
}

// ---------------------------------------------------------------------------
// pack + dt partial maxima
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kDtThreads)
pack_dt_kernel(const fvh_mesh_view m, const fvh_state_view s, workspace w, double *partial) {
  // writes w.pack, the input of the predictor
  float dt_inv = 0.f;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.num_cells;
       c += gridDim.x * blockDim.x) {
    float v[D];
#pragma unroll
    for (int i = 0; i < D; ++i) v[i] = (float)s.velocity[i][c];
    const float a = (float)s.sound_speed[c];
    store_pack<D>(w.pack, c, (float)s.density[c], v, (float)s.pressure[c],
                  (float)s.internal_energy[c], a);
    const float iv = (float)w.inv_vol[c];
    const int q0 = m.cell_face_offsets[c], q1 = m.cell_face_offsets[c + 1];
    for (int q = q0; q < q1; ++q) {
      int f = m.cell_faces[q];
      f = f < 0 ? ~f : f;
      float n[D], area;
      face_geo<D>(w, f, n, area);
      const float dti = (a + fabsf(phys::dot<float, D>(v, n))) * (area * iv);
      dt_inv = smax(dti, dt_inv);
    }
  }
  const double m_ = block_max((double)dt_inv);
  if (threadIdx.x == 0) partial[blockIdx.x] = m_;
}

__global__ void __launch_bounds__(kDtThreads)
dt_final_kernel(const double *partial, int nblocks, fvh_params p, const double *soln_time,
                double *dt_out, fvh_device_status *status) {
  double dt_inv = 0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) dt_inv = smax(partial[i], dt_inv);
  dt_inv = block_max(dt_inv);
  if (threadIdx.x == 0) {
    const double max_dt = p.final_time - soln_time[0];
    if (dt_inv <= 0) {
      atomicMin(status, status_key(0, FVH_ERR_INFINITE_DT));
      dt_out[0] = 0;
    } else {
      double time_step = 1 / dt_inv;
      time_step *= p.cfl;
      dt_out[0] = smin(time_step, max_dt);
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 gradients + Barth-Jespersen vertex limiter
// ---------------------------------------------------------------------------
template <int D, bool LIMIT>
__global__ void __launch_bounds__(kCellThreads)
gradients_kernel(const fvh_mesh_view m, workspace w, const float4 *__restrict__ pk) {
  constexpr int NV = D + 4;
  constexpr float tol = 1.e-9f;
  const int c0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (c0 >= m.num_cells) return;
  float xh[3], xl[3];
  load_cen<D>(w.ccen, c0, xh, xl);
  float u0[NV], umin[NV], umax[NV];
  {
    const prim<float, D> p = load_pack<D>(pk, c0);
    int k = 0;
    u0[k++] = p.d;
#pragma unroll
    for (int d = 0; d < D; ++d) u0[k++] = p.v[d];
    u0[k++] = p.e;
    u0[k++] = p.p;
    u0[k++] = p.a;
  }
#pragma unroll
  for (int k = 0; k < NV; ++k) umin[k] = umax[k] = u0[k];
  float M[6] = {0, 0, 0, 0, 0, 0};
  float b[NV][D];
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int j = 0; j < D; ++j) b[k][j] = 0.f;
  const int q0 = m.cell_nbr_offsets[c0], q1 = m.cell_nbr_offsets[c0 + 1];
  for (int q = q0; q < q1; ++q) {
    const int c1 = m.cell_nbrs[q];
    const prim<float, D> p = load_pack<D>(pk, c1);
    float u1[NV];
    {
      int k = 0;
      u1[k++] = p.d;
#pragma unroll
      for (int d = 0; d < D; ++d) u1[k++] = p.v[d];
      u1[k++] = p.e;
      u1[k++] = p.p;
      u1[k++] = p.a;
    }
    float yh[3], yl[3], dx[3];
    load_cen<D>(w.ccen, c1, yh, yl);
#pragma unroll
    for (int i = 0; i < D; ++i) dx[i] = (yh[i] - xh[i]) + (yl[i] - xl[i]);
    if (D == 2) {
      M[0] += dx[0] * dx[0];
      M[1] += dx[0] * dx[1];
      M[2] += dx[1] * dx[1];
    } else {
      M[0] += dx[0] * dx[0];
      M[1] += dx[0] * dx[1];
      M[2] += dx[0] * dx[D - 1];
      M[3] += dx[1] * dx[1];
      M[4] += dx[1] * dx[D - 1];
      M[5] += dx[D - 1] * dx[D - 1];
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      umin[k] = fminf(u1[k], umin[k]);
      umax[k] = fmaxf(u1[k], umax[k]);
      const float du = u1[k] - u0[k];
#pragma unroll
      for (int j = 0; j < D; ++j) b[k][j] += du * dx[j];
    }
  }
  float g[NV][D];
  if (D == 2) {
    const float det = M[0] * M[2] - M[1] * M[1];
    const float inv = 1.f / det;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      g[k][0] = (b[k][0] * M[2] - b[k][1] * M[1]) * inv;
      g[k][1] = (b[k][1] * M[0] - b[k][0] * M[1]) * inv;
    }
  } else {
    const float a00 = M[0], a01 = M[1], a02 = M[2], a11 = M[3], a12 = M[4], a22 = M[5];
    const float c00 = a11 * a22 - a12 * a12;
    const float c01 = a02 * a12 - a01 * a22;
    const float c02 = a01 * a12 - a02 * a11;
    const float c11 = a00 * a22 - a02 * a02;
    const float c12 = a01 * a02 - a00 * a12;
    const float c22 = a00 * a11 - a01 * a01;
    const float inv = 1.f / (a00 * c00 + a01 * c01 + a02 * c02);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const float b0 = b[k][0], b1 = b[k][1], b2 = b[k][D - 1];
      g[k][0] = (c00 * b0 + c01 * b1 + c02 * b2) * inv;
      g[k][1] = (c01 * b0 + c11 * b1 + c12 * b2) * inv;
      g[k][D - 1] = (c02 * b0 + c12 * b1 + c22 * b2) * inv;
    }
  }
  if (LIMIT) {
    float dpos[NV], dneg[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) dpos[k] = dneg[k] = 0.f;
    const int r0 = m.cell_vertex_offsets[c0], r1 = m.cell_vertex_offsets[c0 + 1];
    for (int r = r0; r < r1; ++r) {
      const int vtx = m.cell_vertices[r];
      float vh[3], vl[3], dxv[3];
      load_cen<D>(w.vcoord, vtx, vh, vl);
#pragma unroll
      for (int i = 0; i < D; ++i) dxv[i] = (vh[i] - xh[i]) + (vl[i] - xl[i]);
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        float du = 0.f;
#pragma unroll
        for (int i = 0; i < D; ++i) du += dxv[i] * g[k][i];
        dpos[k] = fmaxf(du, dpos[k]);
        dneg[k] = fminf(du, dneg[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      float phi = 1.f;
      if (dpos[k] > tol) phi = fminf(phi, __fdividef(umax[k] - u0[k], dpos[k]));
      if (dneg[k] < -tol) phi = fminf(phi, __fdividef(umin[k] - u0[k], dneg[k]));
      phi = fmaxf(phi, 0.f);
#pragma unroll
      for (int i = 0; i < D; ++i) g[k][i] *= phi;
    }
  }
  constexpr int G4 = layout<D>::GRAD4;
  float flat[4 * G4];
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int i = 0; i < D; ++i) flat[k * D + i] = g[k][i];
#pragma unroll
  for (int q = NV * D; q < 4 * G4; ++q) flat[q] = 0.f;
#pragma unroll
  for (int q = 0; q < G4; ++q)
    w.grads[(size_t)G4 * c0 + q] =
        make_float4(flat[4 * q], flat[4 * q + 1], flat[4 * q + 2], flat[4 * q + 3]);
}

// ---------------------------------------------------------------------------
// cell-centric flux + FP64 update
// ---------------------------------------------------------------------------
// reconstruct the state of cell c at offset dx (x_f - x_c) from pack + grads
template <int D, bool SECOND>
__device__ __forceinline__ prim<float, D> recon(const workspace &w, const float4 *pk, int c,
                                                const float *dx, bool swap) {
  prim<float, D> u = load_pack<D>(pk, c);
  if (SECOND) {
    float g[4 * layout<D>::GRAD4];
    load_grads<D>(w.grads, c, g);
    // gradient rows: 0 d, 1..D v, D+1 e, D+2 p, D+3 a
    const int ge = swap ? D + 2 : D + 1;  // row added to the energy slot
    const int gp = swap ? D + 1 : D + 2;  // row added to the pressure slot
#pragma unroll
    for (int i = 0; i < D; ++i) {
      u.d += dx[i] * g[0 * D + i];
#pragma unroll
      for (int d = 0; d < D; ++d) u.v[d] += dx[i] * g[(1 + d) * D + i];
      u.p += dx[i] * g[gp * D + i];
      u.e += dx[i] * g[ge * D + i];
      u.a += dx[i] * g[(D + 3) * D + i];
    }
  }
  return u;
}

template <int D, int KIND, bool SECOND>
__global__ void __launch_bounds__(kCellThreads)
flux_update_kernel(const fvh_mesh_view m, const fvh_state_view s, workspace w,
                   const float4 *__restrict__ pk_in, float4 *__restrict__ pk_out, const double *dt,
                   double factor, double gamma, double cv, int swap, int outflow,
                   double *soln_time, fvh_device_status *status) {
  // Reads only pk_in (all cells) and the cell's own FP64 state; writes the
  // cell's FP64 state and its pk_out record (null after the corrector).
  const double delta_t = dt[0] * factor;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c == 0) soln_time[0] = soln_time[0] + delta_t;
  if (c >= m.num_cells) return;
  double du[D + 2];
#pragma unroll
  for (int k = 0; k < D + 2; ++k) du[k] = 0.0;
  const int q0 = m.cell_face_offsets[c], q1 = m.cell_face_offsets[c + 1];
  for (int q = q0; q < q1; ++q) {
    const int sf = m.cell_faces[q];
    const int f = sf < 0 ? ~sf : sf;
    const int2 cc = reinterpret_cast<const int2 *>(m.face_cells)[f];
    float n[D], area;
    face_geo<D>(w, f, n, area);
    float dx0[D], dx1[D];
    if (D == 2) {
      const float4 t = w.fdx[f];
      dx0[0] = t.x; dx0[1] = t.y; dx1[0] = t.z; dx1[1] = t.w;
    } else {
      const float4 a = w.fdx[2 * (size_t)f], b = w.fdx[2 * (size_t)f + 1];
      dx0[0] = a.x; dx0[1] = a.y; dx0[D - 1] = a.z;
      dx1[0] = b.x; dx1[1] = b.y; dx1[D - 1] = b.z;
    }
    // always evaluated in the face's own orientation (cells(f)[0] -> [1])
    const prim<float, D> wl = recon<D, SECOND>(w, pk_in, cc.x, dx0, swap != 0);
    float F[D + 2];
    if (cc.y >= 0) {
      const prim<float, D> wr = recon<D, SECOND>(w, pk_in, cc.y, dx1, swap != 0);
      phys::riemann<float, D, KIND>(wl, wr, n, F);
    } else if (outflow) {
      phys::phys_flux<float, D>(wl, n, F);
    } else {
      phys::wall<float, D>(wl, n, F);
    }
    if (sf >= 0) {
#pragma unroll
      for (int k = 0; k < D + 2; ++k) du[k] -= (double)(F[k] * area);
    } else {
#pragma unroll
      for (int k = 0; k < D + 2; ++k) du[k] += (double)(F[k] * area);
    }
  }
  const double scale = delta_t * w.inv_vol[c];
  double vel[D];
#pragma unroll
  for (int i = 0; i < D; ++i) vel[i] = s.velocity[i][c];
  const double den0 = s.density[c];
  const double mass = den0 + du[0] * scale;
  double ke = 0.0;
#pragma unroll
  for (int i = 0; i < D; ++i) ke += vel[i] * vel[i];
  const double ener = den0 * (s.internal_energy[c] + 0.5 * ke) + du[D + 1] * scale;
  // 1/mass: FP32 estimate refined by one Newton step in FP64
  double inv_mass = (double)(1.0f / (float)mass);
  inv_mass = inv_mass * (2.0 - mass * inv_mass);
  ke = 0.0;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    vel[i] = (den0 * vel[i] + du[1 + i] * scale) * inv_mass;
    ke += vel[i] * vel[i];
  }
  const double e = ener * inv_mass - 0.5 * ke;
  const double p = (gamma - 1.0) * mass * e;
  const float a = sqrtf((float)(gamma * (gamma - 1.0)) * (float)e);
  s.density[c] = mass;
#pragma unroll
  for (int i = 0; i < D; ++i) s.velocity[i][c] = vel[i];
  s.internal_energy[c] = e;
  s.pressure[c] = p;
  s.temperature[c] = e * (1.0 / cv);
  s.sound_speed[c] = (double)a;
  if (pk_out) {
    float vf[D];
#pragma unroll
    for (int i = 0; i < D; ++i) vf[i] = (float)vel[i];
    store_pack<D>(pk_out, c, (float)mass, vf, (float)p, (float)e, a);
  }
  if (e < 0 || mass < 0) atomicMin(status, status_key(c, FVH_ERR_NEGATIVE_STATE));
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <int D>
static size_t bytes_for(int nc, int nf, int nv) {
  using L = layout<D>;
  return sizeof(float4) * ((size_t)nc * (2 * L::PACK4 + L::GRAD4 + L::CEN4) + (size_t)nv * L::CEN4 +
                           (size_t)nf * (L::FGEO4 + L::FDX4)) +
         sizeof(double) * (size_t)nc + 256 * 8;
}

template <int D>
static void carve(workspace *w) {
  using L = layout<D>;
  char *b = static_cast<char *>(w->base);
  auto take = [&](size_t bytes) {
    char *r = b;
    b += (bytes + 255) / 256 * 256;
    return r;
  };
  w->pack = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nc * L::PACK4));
  w->pack2 = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nc * L::PACK4));
  w->grads = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nc * L::GRAD4));
  w->ccen = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nc * L::CEN4));
  w->vcoord = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nv * L::CEN4));
  w->fgeo = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nf * L::FGEO4));
  w->fdx = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nf * L::FDX4));
  w->inv_vol = reinterpret_cast<double *>(take(sizeof(double) * (size_t)w->nc));
}

template <int D>
static cudaError_t setup(const fvh_mesh_view &m, workspace *w) {
  carve<D>(w);
  const int t = 256;
  setup_cells<D><<<(m.num_cells + t - 1) / t, t>>>(m, *w);
  setup_vertices<D><<<(m.num_vertices + t - 1) / t, t>>>(m, *w);
  setup_faces<D><<<(m.num_faces + t - 1) / t, t>>>(m, *w);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return e;
}

fvh_status create(const fvh_mesh_view &m, const fvh_params &p, workspace **out) {
  *out = nullptr;
  workspace *w = new (std::nothrow) workspace();
  if (!w) return FVH_ERR_OUT_OF_MEMORY;
  w->dim = m.dim;
  w->nc = m.num_cells;
  w->nf = m.num_faces;
  w->nv = m.num_vertices;
  const size_t bytes = m.dim == 2 ? bytes_for<2>(w->nc, w->nf, w->nv)
                                  : bytes_for<3>(w->nc, w->nf, w->nv);
  cudaError_t e = cudaMalloc(&w->base, bytes);
  if (e == cudaSuccess) e = cudaMemset(w->base, 0, bytes);
  if (e == cudaSuccess) e = m.dim == 2 ? setup<2>(m, w) : setup<3>(m, w);
  if (e != cudaSuccess) {
    destroy(w);
    return e == cudaErrorMemoryAllocation ? FVH_ERR_OUT_OF_MEMORY : FVH_ERR_CUDA;
  }
  (void)p;
  *out = w;
  return FVH_OK;
}

void destroy(workspace *w) {
  if (!w) return;
  cudaFree(w->base);
  delete w;
}

template <int D, int KIND, bool SECOND>
static void launch_stage(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                         const fvh_state_view &s, double *t, const double *dt, int stage,
                         fvh_device_status *status, cudaStream_t st, const launch_mark &mark) {
  const int nb = (m.num_cells + kCellThreads - 1) / kCellThreads;
  const float4 *pk_in = stage == 0 ? w->pack : w->pack2;
  float4 *pk_out = stage == 0 ? w->pack2 : nullptr;
  if (SECOND) {
    if (p.limiter == FVH_LIMITER_NONE)
      gradients_kernel<D, false><<<nb, kCellThreads, 0, st>>>(m, *w, pk_in);
    else
      gradients_kernel<D, true><<<nb, kCellThreads, 0, st>>>(m, *w, pk_in);
    mark("gradients");
  }
  flux_update_kernel<D, KIND, SECOND><<<nb, kCellThreads, 0, st>>>(
      m, s, *w, pk_in, pk_out, dt, 0.5, p.gamma, p.cv, p.recon_swap_ep, p.boundary, t, status);
  mark("flux_update");
}

template <int D, int KIND>
static void launch_stage_k(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                           const fvh_state_view &s, double *t, const double *dt, int stage,
                           fvh_device_status *status, cudaStream_t st, const launch_mark &mark) {
  if (p.order == 1)
    launch_stage<D, KIND, false>(w, m, p, s, t, dt, stage, status, st, mark);
  else
    launch_stage<D, KIND, true>(w, m, p, s, t, dt, stage, status, st, mark);
}

template <int D>
static cudaError_t step_d(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                          const fvh_state_view &s, double *t, double *dt, double *partial,
                          int dt_blocks, fvh_device_status *status, cudaStream_t st,
                          const launch_mark &mark) {
  pack_dt_kernel<D><<<dt_blocks, kDtThreads, 0, st>>>(m, s, *w, partial);
  mark("pack_dt");
  dt_final_kernel<<<1, kDtThreads, 0, st>>>(partial, dt_blocks, p, t, dt, status);
  mark("dt_final");
  for (int stage = 0; stage < 2; ++stage) {
    if (p.flux_kind == FVH_FLUX_RUSANOV)
      launch_stage_k<D, FVH_FLUX_RUSANOV>(w, m, p, s, t, dt, stage, status, st, mark);
    else if (p.flux_kind == FVH_FLUX_HLLC)
      launch_stage_k<D, FVH_FLUX_HLLC>(w, m, p, s, t, dt, stage, status, st, mark);
    else
      launch_stage_k<D, FVH_FLUX_HLLE>(w, m, p, s, t, dt, stage, status, st, mark);
  }
  return cudaGetLastError();
}

cudaError_t step(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                 const fvh_state_view &s, double *soln_time, double *dt, double *partial,
                 int dt_blocks, fvh_device_status *status, cudaStream_t st,
                 const launch_mark &mark) {
  return m.dim == 2 ? step_d<2>(w, m, p, s, soln_time, dt, partial, dt_blocks, status, st, mark)
                    : step_d<3>(w, m, p, s, soln_time, dt, partial, dt_blocks, status, st, mark);
}

int launches_per_step(const fvh_params &p) { return p.order == 1 ? 4 : 6; }

}  // namespace mixed
}  // namespace fvh
