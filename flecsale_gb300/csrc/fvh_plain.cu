// Plain FP64 kernels of the Eulerian hydro step (sm_103a).
//
// This translation unit is compiled with --fmad=false: every multiply and add
// below rounds separately, in the order the reference writes them, so the
// results are bit-identical to the reference arithmetic of
//   evaluate_time_step  apps/hydro/tasks.h:331-376
//   evaluate_gradients  apps/hydro/tasks.h:145-321
//   evaluate_fluxes     apps/hydro/tasks.h:385-464
//   apply_update        apps/hydro/tasks.h:589-659
// with the physics of flecsale/eqns/euler_eqns.h and flecsale/eqns/flux.h and
// the ideal gas of flecsale/eos/ideal_gas.h (IEEE division and square root are
// correctly rounded on both CPU and GPU).
//
// Layout: every field component is its own FP64 plane (SoA), so a warp's 32
// consecutive cells or faces read 256 contiguous bytes per plane.  Neighbour
// gathers follow the CSR lists in the reference's iteration order; with
// lexicographic numbering the neighbours of a warp's cells share cache lines and
// are served from L1/L2 after the first touch.
#include <cuda_runtime.h>

#include <cstdint>

#include "flecsale_gb300.h"
#include "fvh_kernels.h"

namespace fvh {
namespace plain {

// std::max / std::min semantics of the reference (a < b ? b : a)
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }

template <int D>
__device__ __forceinline__ double dot(const double *a, const double *b) {
  double s = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) s += a[i] * b[i];
  return s;
}

// Same slots as pack_copy(c, d, v, p, e, T, a) (tasks.h:420).  T is carried by
// the reference but never used in a flux, so it is not loaded here.
template <int D>
struct prim {
  double d, v[D], p, e, a;
};

template <int D>
__device__ __forceinline__ double total_energy(const prim<D> &u) {
  return u.e + 0.5 * dot<D>(u.v, u.v);
}

template <int D>
__device__ __forceinline__ void phys_flux(const prim<D> &u, const double *n, double *f) {
  const double et = total_energy<D>(u);
  const double vn = dot<D>(u.v, n);
  const double mass_flux = u.d * vn;
  f[0] = mass_flux;
#pragma unroll
  for (int i = 0; i < D; ++i) f[1 + i] = mass_flux * u.v[i] + u.p * n[i];
  f[D + 1] = mass_flux * (et + u.p / u.d);
}

template <int D>
__device__ __forceinline__ void solution_delta(const prim<D> &l, const prim<D> &r,
                                               double *du) {
  const double ener_l = l.d * total_energy<D>(l);
  const double ener_r = r.d * total_energy<D>(r);
  du[0] = r.d - l.d;
#pragma unroll
  for (int i = 0; i < D; ++i) du[1 + i] = r.d * r.v[i] - l.d * l.v[i];
  du[D + 1] = ener_r - ener_l;
}

template <int D>
__device__ __forceinline__ void hlle(const prim<D> &l, const prim<D> &r,
                                     const double *n, double *f) {
  const double vnl = dot<D>(l.v, n), vnr = dot<D>(r.v, n);
  const double lambda_l = smin(vnl - l.a, vnr - r.a);
  const double lambda_r = smax(vnl + l.a, vnr + r.a);
  if (lambda_l >= 0) {
    phys_flux<D>(l, n, f);
  } else if (lambda_r <= 0) {
    phys_flux<D>(r, n, f);
  } else {
    double fl[D + 2], fr[D + 2], du[D + 2];
    phys_flux<D>(l, n, fl);
    phys_flux<D>(r, n, fr);
    const double c1 = lambda_l * lambda_r;
    const double c2 = lambda_r - lambda_l;
    const double c2inv = 1 / c2;
    solution_delta<D>(l, r, du);
#pragma unroll
    for (int i = 0; i < D + 2; ++i)
      f[i] = c2inv * (lambda_r * fl[i] - lambda_l * fr[i] + c1 * du[i]);
  }
}

template <int D>
__device__ __forceinline__ void rusanov(const prim<D> &l, const prim<D> &r,
                                        const double *n, double *f) {
  double fl[D + 2], fr[D + 2], du[D + 2];
  phys_flux<D>(l, n, fl);
  phys_flux<D>(r, n, fr);
  const double sl = l.a + fabs(dot<D>(l.v, n));
  const double sr = r.a + fabs(dot<D>(r.v, n));
  const double s = smax(sl, sr);
  solution_delta<D>(l, r, du);
  const double half_s = s / 2;
#pragma unroll
  for (int i = 0; i < D + 2; ++i) f[i] = (fl[i] + fr[i]) / 2 - du[i] * half_s;
}

// Toro's HLLC (sec. 10.4) with the hlle_flux wave-speed estimates.
template <int D>
__device__ __forceinline__ void hllc(const prim<D> &l, const prim<D> &r,
                                     const double *n, double *f) {
  const double vnl = dot<D>(l.v, n), vnr = dot<D>(r.v, n);
  const double sL = smin(vnl - l.a, vnr - r.a);
  const double sR = smax(vnl + l.a, vnr + r.a);
  if (sL >= 0) {
    phys_flux<D>(l, n, f);
    return;
  }
  if (sR <= 0) {
    phys_flux<D>(r, n, f);
    return;
  }
  const double ml = l.d * (sL - vnl);
  const double mr = r.d * (sR - vnr);
  const double sM = (r.p - l.p + ml * vnl - mr * vnr) / (ml - mr);
  const bool left = sM >= 0;
  const prim<D> &u = left ? l : r;
  const double sK = left ? sL : sR;
  const double mK = left ? ml : mr;
  const double vnK = left ? vnl : vnr;
  double fk[D + 2];
  phys_flux<D>(u, n, fk);
  const double EK = u.d * total_energy<D>(u);
  const double fac = mK / (sK - sM);
  const double dvn = sM - vnK;
  f[0] = fk[0] + sK * (fac - u.d);
#pragma unroll
  for (int i = 0; i < D; ++i)
    f[1 + i] = fk[1 + i] + sK * (fac * (u.v[i] + dvn * n[i]) - u.d * u.v[i]);
  f[D + 1] = fk[D + 1] + sK * (fac * (EK / u.d + dvn * (sM + u.p / mK)) - EK);
}

// ---------------------------------------------------------------------------
// Order-preserving integer keys of doubles.  Comparisons, minima and maxima of
// doubles run on the integer pipe through these keys (the FP64 pipe of this
// chip is narrow).  key(a) < key(b) exactly when a < b for non-NaN values;
// -0 and +0 share the key of +0, so a minimum or maximum can differ from the
// floating-point one only in the sign of a zero.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long okey(double x) {
  long long b = __double_as_longlong(x);
  b = (b == (long long)0x8000000000000000ull) ? 0ll : b;
  return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
__device__ __forceinline__ double from_okey(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffll));
}

// ---------------------------------------------------------------------------
// dt: per-block maxima of (a + |v.n|) / (V/A), then one block finishes.
// With PRE the V/A of each (cell, face) slot comes from a table built once per
// mesh by the same division.
// ---------------------------------------------------------------------------
template <int D, bool PRE>
__global__ void __launch_bounds__(kDtThreads)
dt_partial_kernel(const fvh_mesh_view m, const fvh_state_view s, double *partial,
                  const double *__restrict__ slot_dx) {
  double dt_inv = 0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.num_cells;
       c += gridDim.x * blockDim.x) {
    double v[D];
#pragma unroll
    for (int i = 0; i < D; ++i) v[i] = s.velocity[i][c];
    const double a = s.sound_speed[c];
    const double vol = PRE ? 0.0 : m.cell_volume[c];
    const int q0 = m.cell_face_offsets[c], q1 = m.cell_face_offsets[c + 1];
    for (int q = q0; q < q1; ++q) {
      int f = m.cell_faces[q];
      f = f < 0 ? ~f : f;
      double n[D];
#pragma unroll
      for (int i = 0; i < D; ++i) n[i] = m.face_normal[i][f];
      const double delta_x = PRE ? slot_dx[q] : vol / m.face_area[f];
      const double dti = (a + fabs(dot<D>(v, n))) / delta_x;
      dt_inv = smax(dti, dt_inv);
    }
  }
  dt_inv = block_max(dt_inv);
  if (threadIdx.x == 0) partial[blockIdx.x] = dt_inv;
}

__global__ void __launch_bounds__(kDtThreads)
dt_final_kernel(const double *partial, int nblocks, fvh_params p,
                const double *soln_time, double *dt_out, fvh_device_status *status) {
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
// Geometry-only tables built once per mesh for the solver (same operations in
// the same order as the on-the-fly code, so the values are identical).
// ---------------------------------------------------------------------------
template <int D>
__global__ void slot_dx_kernel(const fvh_mesh_view m, double *slot_dx) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.num_cells) return;
  const double vol = m.cell_volume[c];
  for (int q = m.cell_face_offsets[c]; q < m.cell_face_offsets[c + 1]; ++q) {
    int f = m.cell_faces[q];
    f = f < 0 ? ~f : f;
    slot_dx[q] = vol / m.face_area[f];
  }
}

// lsq record per cell: 2D (a00 a01 a11 denom); 3D (a00 a01 a02 a11 a12 a22
// min1 min2 min3 denom), tasks.h:210-228 and :250-261
template <int D>
struct lsq_width {
  static constexpr int value = D == 2 ? 4 : 10;
};

template <int D>
__device__ __forceinline__ void lsq_matrix(const fvh_mesh_view &m, int c0, double *r) {
  double x0[D];
#pragma unroll
  for (int i = 0; i < D; ++i) x0[i] = m.cell_centroid[i][c0];
  double dxdx[6] = {0, 0, 0, 0, 0, 0};
  for (int q = m.cell_nbr_offsets[c0]; q < m.cell_nbr_offsets[c0 + 1]; ++q) {
    const int c1 = m.cell_nbrs[q];
    double dx[D];
#pragma unroll
    for (int d = 0; d < D; ++d) dx[d] = m.cell_centroid[d][c1] - x0[d];
    if (D == 2) {
      dxdx[0] += dx[0] * dx[0];
      dxdx[1] += dx[0] * dx[1];
      dxdx[2] += dx[1] * dx[1];
    } else {
      dxdx[0] += dx[0] * dx[0];
      dxdx[1] += dx[0] * dx[1];
      dxdx[2] += dx[0] * dx[D - 1];
      dxdx[3] += dx[1] * dx[1];
      dxdx[4] += dx[1] * dx[D - 1];
      dxdx[5] += dx[D - 1] * dx[D - 1];
    }
  }
  if (D == 2) {
    r[0] = dxdx[0];
    r[1] = dxdx[1];
    r[2] = dxdx[2];
    r[3] = 1 / (dxdx[0] * dxdx[2] - dxdx[1] * dxdx[1]);
  } else {
    const double a00 = dxdx[0], a01 = dxdx[1], a02 = dxdx[2], a11 = dxdx[3],
                 a12 = dxdx[4], a22 = dxdx[5];
    const double min1 = a11 * a22 - a12 * a12;
    const double min2 = a01 * a22 - a12 * a02;
    const double min3 = a01 * a12 - a11 * a02;
    for (int k = 0; k < 6; ++k) r[k] = dxdx[k];
    r[6] = min1;
    r[7] = min2;
    r[8] = min3;
    r[9] = 1 / (a00 * min1 - a01 * min2 + a02 * min3);
  }
}

template <int D>
__global__ void lsq_kernel(const fvh_mesh_view m, double *lsq) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.num_cells) return;
  constexpr int W = lsq_width<D>::value;
  double r[W];
  lsq_matrix<D>(m, c, r);
#pragma unroll
  for (int k = 0; k < W; ++k) lsq[(size_t)k * m.num_cells + c] = r[k];
}

// ---------------------------------------------------------------------------
// gradients + Barth-Jespersen vertex limiter (tasks.h:145-321)
// With PRE the geometry-only matrix terms come from the lsq table.
// ---------------------------------------------------------------------------
template <int D, bool LIMIT, bool PRE>
__global__ void __launch_bounds__(kCellThreads)
gradients_kernel(const fvh_mesh_view m, const fvh_state_view s, const fvh_gradient_view g,
                 const double *__restrict__ lsq) {
  constexpr int NV = D + 4;
  constexpr int W = lsq_width<D>::value;
  constexpr double tol = 1.e-9;
  const int c0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (c0 >= m.num_cells) return;
  double x0[D];
#pragma unroll
  for (int i = 0; i < D; ++i) x0[i] = m.cell_centroid[i][c0];
  double u0[NV];
  long long kmin[NV], kmax[NV];  // umin / umax as order keys
  {
    int i = 0;
    u0[i++] = s.density[c0];
#pragma unroll
    for (int d = 0; d < D; ++d) u0[i++] = s.velocity[d][c0];
    u0[i++] = s.internal_energy[c0];
    u0[i++] = s.pressure[c0];
    u0[i++] = s.sound_speed[c0];
  }
#pragma unroll
  for (int k = 0; k < NV; ++k) kmin[k] = kmax[k] = okey(u0[k]);
  double dudx[NV][D];
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int j = 0; j < D; ++j) dudx[k][j] = 0;
  const int q0 = m.cell_nbr_offsets[c0], q1 = m.cell_nbr_offsets[c0 + 1];
  for (int q = q0; q < q1; ++q) {
    const int c1 = m.cell_nbrs[q];
    double u1[NV];
    {
      int i = 0;
      u1[i++] = s.density[c1];
#pragma unroll
      for (int d = 0; d < D; ++d) u1[i++] = s.velocity[d][c1];
      u1[i++] = s.internal_energy[c1];
      u1[i++] = s.pressure[c1];
      u1[i++] = s.sound_speed[c1];
    }
    double dx[D];
#pragma unroll
    for (int d = 0; d < D; ++d) dx[d] = m.cell_centroid[d][c1] - x0[d];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const long long k1 = okey(u1[k]);
      kmin[k] = (k1 < kmin[k]) ? k1 : kmin[k];  // std::min(u1, umin)
      kmax[k] = (kmax[k] < k1) ? k1 : kmax[k];  // std::max(u1, umax)
      const double du = u1[k] - u0[k];
#pragma unroll
      for (int j = 0; j < D; ++j) dudx[k][j] += du * dx[j];
    }
  }
  double r[W];
  if (PRE) {
#pragma unroll
    for (int k = 0; k < W; ++k) r[k] = lsq[(size_t)k * m.num_cells + c0];
  } else {
    lsq_matrix<D>(m, c0, r);
  }
  double gu[NV][D];
  if (D == 2) {
    const double a00 = r[0], a01 = r[1], a11 = r[2], denom = r[3];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      gu[k][0] = (dudx[k][0] * a11 - dudx[k][1] * a01) * denom;
      gu[k][1] = (dudx[k][1] * a00 - dudx[k][0] * a01) * denom;
    }
  } else {
    const double a00 = r[0], a01 = r[1], a02 = r[2], a11 = r[3], a12 = r[4], a22 = r[5];
    const double min1 = r[6], min2 = r[7], min3 = r[W - 2], denom = r[W - 1];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double b0 = dudx[k][0], b1 = dudx[k][1], b2 = dudx[k][D - 1];
      gu[k][0] = (b0 * min1 - a01 * (b1 * a22 - a12 * b2) + a02 * (b1 * a12 - a11 * b2)) * denom;
      gu[k][1] = (a00 * (b1 * a22 - a12 * b2) - b0 * min2 + a02 * (b2 * a01 - a02 * b1)) * denom;
      gu[k][D - 1] = (a00 * (b2 * a11 - a12 * b1) - a01 * (b2 * a01 - a02 * b1) + b0 * min3) * denom;
    }
  }
  if (LIMIT) {
    // phi_k = min over vertices of (umax-u0)/du or (umin-u0)/du.  Correctly
    // rounded division is monotone in the divisor, so for each variable only
    // the largest du > tol and the smallest du < -tol can set the minimum; the
    // result equals the reference's per-vertex minimum.
    const long long ktol = okey(tol), kntol = okey(-tol);
    long long kpos[NV], kneg[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) kpos[k] = kneg[k] = 0;
    const int r0 = m.cell_vertex_offsets[c0], r1 = m.cell_vertex_offsets[c0 + 1];
    for (int rr = r0; rr < r1; ++rr) {
      const int vtx = m.cell_vertices[rr];
      double dxv[D];
#pragma unroll
      for (int i = 0; i < D; ++i) dxv[i] = m.vertex_coord[i][vtx] - x0[i];
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        double u1 = u0[k];
#pragma unroll
        for (int i = 0; i < D; ++i) u1 += dxv[i] * gu[k][i];
        const long long kd = okey(u1 - u0[k]);
        if (kd > ktol) kpos[k] = (kpos[k] < kd) ? kd : kpos[k];
        else if (kd < kntol) kneg[k] = (kd < kneg[k]) ? kd : kneg[k];
      }
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      long long kphi = okey(1.0);
      if (kpos[k] > ktol) {
        const long long kq = okey((from_okey(kmax[k]) - u0[k]) / from_okey(kpos[k]));
        kphi = (kq < kphi) ? kq : kphi;
      }
      if (kneg[k] < kntol) {
        const long long kq = okey((from_okey(kmin[k]) - u0[k]) / from_okey(kneg[k]));
        kphi = (kq < kphi) ? kq : kphi;
      }
      kphi = (kphi < 0) ? 0 : kphi;  // std::max(phi, 0)
      if (kphi != okey(1.0)) {
        const double phi = from_okey(kphi);
#pragma unroll
        for (int i = 0; i < D; ++i) gu[k][i] *= phi;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < D; ++i) {
    int k = 0;
    g.density[i][c0] = gu[k++][i];
#pragma unroll
    for (int d = 0; d < D; ++d) g.velocity[d][i][c0] = gu[k++][i];
    g.internal_energy[i][c0] = gu[k++][i];
    g.pressure[i][c0] = gu[k++][i];
    g.sound_speed[i][c0] = gu[k++][i];
  }
}

// ---------------------------------------------------------------------------
// face fluxes (tasks.h:385-464)
// ---------------------------------------------------------------------------
template <int D, bool SECOND>
__device__ __forceinline__ prim<D> reconstruct(const fvh_mesh_view &m,
                                               const fvh_state_view &s,
                                               const fvh_gradient_view &g, int c,
                                               const double *fx, bool swap) {
  prim<D> w;
  w.d = s.density[c];
#pragma unroll
  for (int i = 0; i < D; ++i) w.v[i] = s.velocity[i][c];
  w.p = s.pressure[c];
  w.e = s.internal_energy[c];
  w.a = s.sound_speed[c];
  if (SECOND) {
    double dx[D];
#pragma unroll
    for (int i = 0; i < D; ++i) dx[i] = fx[i] - m.cell_centroid[i][c];
    double *const *gp = swap ? g.internal_energy : g.pressure;
    double *const *ge = swap ? g.pressure : g.internal_energy;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      w.d += dx[i] * g.density[i][c];
#pragma unroll
      for (int d = 0; d < D; ++d) w.v[d] += dx[i] * g.velocity[d][i][c];
      w.p += dx[i] * gp[i][c];
      w.e += dx[i] * ge[i][c];
      w.a += dx[i] * g.sound_speed[i][c];
    }
  }
  return w;
}

template <int D, int KIND, bool SECOND>
__global__ void __launch_bounds__(kFaceThreads)
fluxes_kernel(const fvh_mesh_view m, const fvh_state_view s, const fvh_gradient_view g,
              const fvh_flux_view fl, int swap, int outflow) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.num_faces) return;
  const int2 cc = reinterpret_cast<const int2 *>(m.face_cells)[f];
  double n[D], fx[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    n[i] = m.face_normal[i][f];
    fx[i] = m.face_centroid[i][f];
  }
  const prim<D> wl = reconstruct<D, SECOND>(m, s, g, cc.x, fx, swap != 0);
  double F[D + 2];
  if (cc.y >= 0) {
    const prim<D> wr = reconstruct<D, SECOND>(m, s, g, cc.y, fx, swap != 0);
    if (KIND == FVH_FLUX_RUSANOV)
      rusanov<D>(wl, wr, n, F);
    else if (KIND == FVH_FLUX_HLLC)
      hllc<D>(wl, wr, n, F);
    else
      hlle<D>(wl, wr, n, F);
  } else if (outflow) {
    phys_flux<D>(wl, n, F);
  } else {
    F[0] = 0;
#pragma unroll
    for (int i = 0; i < D; ++i) F[1 + i] = wl.p * n[i];
    F[D + 1] = 0;
  }
  const double area = m.face_area[f];
  fl.mass[f] = F[0] * area;
#pragma unroll
  for (int i = 0; i < D; ++i) fl.momentum[i][f] = F[1 + i] * area;
  fl.energy[f] = F[D + 1] * area;
}

// ---------------------------------------------------------------------------
// gather + conservative update + EOS (tasks.h:589-659)
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kCellThreads)
update_kernel(const fvh_mesh_view m, const fvh_flux_view fl, const fvh_state_view s,
              const double *dt, double factor, double gamma, double cv,
              double *soln_time, fvh_device_status *status) {
  double delta_t = dt[0];
  delta_t *= factor;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c == 0) soln_time[0] = 0.0 + soln_time[0] + delta_t;
  if (c >= m.num_cells) return;
  double du[D + 2];
#pragma unroll
  for (int k = 0; k < D + 2; ++k) du[k] = 0;
  const int q0 = m.cell_face_offsets[c], q1 = m.cell_face_offsets[c + 1];
  for (int q = q0; q < q1; ++q) {
    const int sf = m.cell_faces[q];
    const int f = sf < 0 ? ~sf : sf;
    double F[D + 2];
    F[0] = fl.mass[f];
#pragma unroll
    for (int i = 0; i < D; ++i) F[1 + i] = fl.momentum[i][f];
    F[D + 1] = fl.energy[f];
    if (sf >= 0) {
#pragma unroll
      for (int k = 0; k < D + 2; ++k) du[k] -= F[k];
    } else {
#pragma unroll
      for (int k = 0; k < D + 2; ++k) du[k] += F[k];
    }
  }
  const double scale = delta_t / m.cell_volume[c];
#pragma unroll
  for (int k = 0; k < D + 2; ++k) du[k] *= scale;
  double vel[D];
#pragma unroll
  for (int i = 0; i < D; ++i) vel[i] = s.velocity[i][c];
  const double den0 = s.density[c];
  const double mass = den0 + du[0];
  const double ener = den0 * (s.internal_energy[c] + 0.5 * dot<D>(vel, vel)) + du[D + 1];
  const double inv_mass = 1 / mass;
#pragma unroll
  for (int i = 0; i < D; ++i) vel[i] = (den0 * vel[i] + du[1 + i]) * inv_mass;
  const double e = ener * inv_mass - 0.5 * dot<D>(vel, vel);
  s.density[c] = mass;
#pragma unroll
  for (int i = 0; i < D; ++i) s.velocity[i][c] = vel[i];
  s.internal_energy[c] = e;
  s.pressure[c] = (gamma - 1.0) * mass * e;
  s.temperature[c] = cv == 1.0 ? e : e / cv;  // x / 1 == x exactly
  s.sound_speed[c] = sqrt(gamma * (gamma - 1.0) * e);
  if (e < 0 || mass < 0) atomicMin(status, status_key(c, FVH_ERR_NEGATIVE_STATE));
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template <int D>
cudaError_t launch_dt(const fvh_mesh_view &m, const fvh_state_view &s,
                      const fvh_params &p, const double *soln_time, double *dt,
                      double *partial, int nblocks, fvh_device_status *status,
                      cudaStream_t st, const double *slot_dx) {
  if (slot_dx)
    dt_partial_kernel<D, true><<<nblocks, kDtThreads, 0, st>>>(m, s, partial, slot_dx);
  else
    dt_partial_kernel<D, false><<<nblocks, kDtThreads, 0, st>>>(m, s, partial, nullptr);
  dt_final_kernel<<<1, kDtThreads, 0, st>>>(partial, nblocks, p, soln_time, dt, status);
  return cudaGetLastError();
}

template <int D>
cudaError_t launch_gradients(const fvh_mesh_view &m, const fvh_state_view &s,
                             const fvh_gradient_view &g, const fvh_params &p,
                             cudaStream_t st, const double *lsq) {
  const int nb = (m.num_cells + kCellThreads - 1) / kCellThreads;
  const bool lim = p.limiter != FVH_LIMITER_NONE;
  if (lsq) {
    if (lim)
      gradients_kernel<D, true, true><<<nb, kCellThreads, 0, st>>>(m, s, g, lsq);
    else
      gradients_kernel<D, false, true><<<nb, kCellThreads, 0, st>>>(m, s, g, lsq);
  } else {
    if (lim)
      gradients_kernel<D, true, false><<<nb, kCellThreads, 0, st>>>(m, s, g, nullptr);
    else
      gradients_kernel<D, false, false><<<nb, kCellThreads, 0, st>>>(m, s, g, nullptr);
  }
  return cudaGetLastError();
}

template <int D>
cudaError_t build_tables(const fvh_mesh_view &m, double *lsq, double *slot_dx) {
  const int t = 128, nb = (m.num_cells + t - 1) / t;
  lsq_kernel<D><<<nb, t>>>(m, lsq);
  slot_dx_kernel<D><<<nb, t>>>(m, slot_dx);
  return cudaGetLastError();
}

int lsq_doubles_per_cell(int dim) { return dim == 2 ? lsq_width<2>::value : lsq_width<3>::value; }

template <int D, bool SECOND>
static void launch_fluxes_kind(const fvh_mesh_view &m, const fvh_state_view &s,
                               const fvh_gradient_view &g, const fvh_flux_view &fl,
                               const fvh_params &p, cudaStream_t st) {
  const int nb = (m.num_faces + kFaceThreads - 1) / kFaceThreads;
  if (p.flux_kind == FVH_FLUX_RUSANOV)
    fluxes_kernel<D, FVH_FLUX_RUSANOV, SECOND><<<nb, kFaceThreads, 0, st>>>(m, s, g, fl, p.recon_swap_ep, p.boundary);
  else if (p.flux_kind == FVH_FLUX_HLLC)
    fluxes_kernel<D, FVH_FLUX_HLLC, SECOND><<<nb, kFaceThreads, 0, st>>>(m, s, g, fl, p.recon_swap_ep, p.boundary);
  else
    fluxes_kernel<D, FVH_FLUX_HLLE, SECOND><<<nb, kFaceThreads, 0, st>>>(m, s, g, fl, p.recon_swap_ep, p.boundary);
}

template <int D>
cudaError_t launch_fluxes(const fvh_mesh_view &m, const fvh_state_view &s,
                          const fvh_gradient_view &g, const fvh_flux_view &fl,
                          const fvh_params &p, cudaStream_t st) {
  if (p.order == 1)
    launch_fluxes_kind<D, false>(m, s, g, fl, p, st);
  else
    launch_fluxes_kind<D, true>(m, s, g, fl, p, st);
  return cudaGetLastError();
}

template <int D>
cudaError_t launch_update(const fvh_mesh_view &m, const fvh_params &p, const double *dt,
                          double factor, const fvh_flux_view &fl,
                          const fvh_state_view &s, double *soln_time,
                          fvh_device_status *status, cudaStream_t st) {
  const int nb = (m.num_cells + kCellThreads - 1) / kCellThreads;
  update_kernel<D><<<nb, kCellThreads, 0, st>>>(m, fl, s, dt, factor, p.gamma, p.cv,
                                                soln_time, status);
  return cudaGetLastError();
}

#define FVH_INSTANTIATE(D)                                                              \
  template cudaError_t launch_dt<D>(const fvh_mesh_view &, const fvh_state_view &,     \
                                    const fvh_params &, const double *, double *,      \
                                    double *, int, fvh_device_status *, cudaStream_t,  \
                                    const double *);                                   \
  template cudaError_t launch_gradients<D>(const fvh_mesh_view &, const fvh_state_view &, \
                                           const fvh_gradient_view &, const fvh_params &, \
                                           cudaStream_t, const double *);              \
  template cudaError_t build_tables<D>(const fvh_mesh_view &, double *, double *);     \
  template cudaError_t launch_fluxes<D>(const fvh_mesh_view &, const fvh_state_view &, \
                                        const fvh_gradient_view &, const fvh_flux_view &, \
                                        const fvh_params &, cudaStream_t);             \
  template cudaError_t launch_update<D>(const fvh_mesh_view &, const fvh_params &,     \
                                        const double *, double, const fvh_flux_view &, \
                                        const fvh_state_view &, double *,              \
                                        fvh_device_status *, cudaStream_t);
FVH_INSTANTIATE(2)
FVH_INSTANTIATE(3)

}  // namespace plain
}  // namespace fvh
