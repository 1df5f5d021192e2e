// ORACLE — test infrastructure only.
//
// A CPU restatement of FleCSALE's Eulerian hydro tasks (apps/hydro) used as the
// checker for the GPU kernels.  Only the tests, the smoke check and the CPU
// baseline leg of the benchmark load it; the product never does.
//
// It follows the reference's arithmetic order statement by statement, so that
// an IEEE FP64 build without floating-point contraction (-ffp-contract=off)
// reproduces the reference's rounding:
//   evaluate_time_step   apps/hydro/tasks.h:331-376
//   evaluate_gradients   apps/hydro/tasks.h:145-321 (gradient_2d/3d :109-143)
//   evaluate_fluxes      apps/hydro/tasks.h:385-464 (owned faces; the shared-cell
//                        loop :467-534 recomputes the same faces on other ranks)
//   apply_update         apps/hydro/tasks.h:589-659, update_soln_time :545-576
//   time loop            apps/hydro/driver.h:317-376
//   physics              flecsale/eqns/euler_eqns.h:167-410, flecsale/eqns/flux.h:51-106
//   equation of state    flecsale/eos/ideal_gas.h:178-226
// The reference's ristra::math::dot_product sums from zero in index order; that
// order is used for every dot product here.
//
// HLLC is not in the reference; the restatement here follows Toro, "Riemann
// Solvers and Numerical Methods for Fluid Dynamics" (3rd ed.), section 10.4,
// with the wave-speed estimates of hlle_flux (flux.h:82-86).  Parity for it is
// against this oracle only.
//
// Pinning: tests/test_oracle_golden.py runs this oracle on the mesh of the
// reference regression test apps/hydro/2d (32x32 quads, 20 steps) and compares
// against shock_box_2d-solution_rank000000.txt.1procs.std with the reference's
// numdiff semantics (absolute 1e-14, cmake/regression.cmake:19).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

#include "flecsale_gb300.h"

namespace {

constexpr int MAXV = 7;  // d, v[3], e, p, a

template <int D>
inline double dot(const double *a, const double *b) {
  double s = 0;
  for (int i = 0; i < D; ++i) s += a[i] * b[i];
  return s;
}

// Primitive state tuple, same slots as pack_copy(c, d, v, p, e, T, a)
// (tasks.h:420, types.h:150-155).
template <int D>
struct prim {
  double d, v[D], p, e, T, a;
};

// euler_eqns_t::total_energy (euler_eqns.h:167-173)
template <int D>
inline double total_energy(const prim<D> &u) {
  return u.e + 0.5 * dot<D>(u.v, u.v);
}

// euler_eqns_t::flux (euler_eqns.h:274-304)
template <int D>
inline void phys_flux(const prim<D> &u, const double *n, double *f) {
  const double et = total_energy<D>(u);
  const double vn = dot<D>(u.v, n);
  const double mass_flux = u.d * vn;
  f[0] = mass_flux;
  for (int i = 0; i < D; ++i) f[1 + i] = mass_flux * u.v[i] + u.p * n[i];
  f[D + 1] = mass_flux * (et + u.p / u.d);
}

// euler_eqns_t::solution_delta (euler_eqns.h:238-265): ur - ul
template <int D>
inline void solution_delta(const prim<D> &l, const prim<D> &r, double *du) {
  const double ener_l = l.d * total_energy<D>(l);
  const double ener_r = r.d * total_energy<D>(r);
  du[0] = r.d - l.d;
  for (int i = 0; i < D; ++i) du[1 + i] = r.d * r.v[i] - l.d * l.v[i];
  du[D + 1] = ener_r - ener_l;
}

// hlle_flux (flux.h:79-106), minmax_eigenvalues (euler_eqns.h:222-230)
template <int D>
inline void hlle(const prim<D> &l, const prim<D> &r, const double *n, double *f) {
  const double vnl = dot<D>(l.v, n), vnr = dot<D>(r.v, n);
  const double sl_first = vnl - l.a, sl_second = vnl + l.a;
  const double sr_first = vnr - r.a, sr_second = vnr + r.a;
  const double lambda_l = std::min(sl_first, sr_first);
  const double lambda_r = std::max(sl_second, sr_second);
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
    for (int i = 0; i < D + 2; ++i)
      f[i] = c2inv * (lambda_r * fl[i] - lambda_l * fr[i] + c1 * du[i]);
  }
}

// rusanov_flux (flux.h:51-65), fastest_wavespeed (euler_eqns.h:183-189)
template <int D>
inline void rusanov(const prim<D> &l, const prim<D> &r, const double *n, double *f) {
  double fl[D + 2], fr[D + 2], du[D + 2];
  phys_flux<D>(l, n, fl);
  phys_flux<D>(r, n, fr);
  const double sl = l.a + std::abs(dot<D>(l.v, n));
  const double sr = r.a + std::abs(dot<D>(r.v, n));
  const double s = std::max(sl, sr);
  solution_delta<D>(l, r, du);
  const double half_s = s / 2;
  for (int i = 0; i < D + 2; ++i) {
    const double favg = (fl[i] + fr[i]) / 2;
    f[i] = favg - du[i] * half_s;
  }
}

// HLLC (Toro sec. 10.4; multi-dimensional star state with the normal velocity
// replaced by the contact speed), wave speeds as hlle_flux.
template <int D>
inline void hllc(const prim<D> &l, const prim<D> &r, const double *n, double *f) {
  const double vnl = dot<D>(l.v, n), vnr = dot<D>(r.v, n);
  const double sL = std::min(vnl - l.a, vnr - r.a);
  const double sR = std::max(vnl + l.a, vnr + r.a);
  if (sL >= 0) {
    phys_flux<D>(l, n, f);
    return;
  }
  if (sR <= 0) {
    phys_flux<D>(r, n, f);
    return;
  }
  const double ml = l.d * (sL - vnl);  // < 0
  const double mr = r.d * (sR - vnr);  // > 0
  const double sM = (r.p - l.p + ml * vnl - mr * vnr) / (ml - mr);
  const bool left = sM >= 0;
  const prim<D> &u = left ? l : r;
  const double sK = left ? sL : sR;
  const double mK = left ? ml : mr;
  const double vnK = left ? vnl : vnr;
  double fk[D + 2];
  phys_flux<D>(u, n, fk);
  const double EK = u.d * total_energy<D>(u);
  const double fac = mK / (sK - sM);          // rho_K (S_K - vn_K) / (S_K - S*)
  const double dvn = sM - vnK;
  double ustar[D + 2], uk[D + 2];
  ustar[0] = fac;
  uk[0] = u.d;
  for (int i = 0; i < D; ++i) {
    ustar[1 + i] = fac * (u.v[i] + dvn * n[i]);
    uk[1 + i] = u.d * u.v[i];
  }
  ustar[D + 1] = fac * (EK / u.d + dvn * (sM + u.p / mK));
  uk[D + 1] = EK;
  for (int i = 0; i < D + 2; ++i) f[i] = fk[i] + sK * (ustar[i] - uk[i]);
}

// wall_flux (euler_eqns.h:313-324) on the reconstructed pressure slot
template <int D>
inline void wall(const prim<D> &u, const double *n, double *f) {
  f[0] = 0;
  for (int i = 0; i < D; ++i) f[1 + i] = u.p * n[i];
  f[D + 1] = 0;
}

template <int D>
double evaluate_time_step(const fvh_mesh_view &m, const fvh_state_view &s,
                          const fvh_params &p, double soln_time, int *status) {
  const double max_dt = p.final_time - soln_time;
  double dt_inv = 0;
#pragma omp parallel for reduction(max : dt_inv) schedule(static)
  for (int c = 0; c < m.num_cells; ++c) {
    double v[D];
    for (int i = 0; i < D; ++i) v[i] = s.velocity[i][c];
    for (int q = m.cell_face_offsets[c]; q < m.cell_face_offsets[c + 1]; ++q) {
      int f = m.cell_faces[q];
      if (f < 0) f = ~f;
      double n[D];
      for (int i = 0; i < D; ++i) n[i] = m.face_normal[i][f];
      const double delta_x = m.cell_volume[c] / m.face_area[f];
      const double ws = s.sound_speed[c] + std::abs(dot<D>(v, n));
      const double dti = ws / delta_x;
      dt_inv = std::max(dti, dt_inv);
    }
  }
  if (dt_inv <= 0) {
    *status = FVH_ERR_INFINITE_DT;
    return 0;
  }
  double time_step = 1 / dt_inv;
  time_step *= p.cfl;
  time_step = std::min(time_step, max_dt);
  *status = FVH_OK;
  return time_step;
}

template <int D>
void evaluate_gradients(const fvh_mesh_view &m, const fvh_state_view &s,
                        const fvh_gradient_view &g, const fvh_params &p) {
  constexpr int NV = D + 4;
  constexpr double tol = 1.e-9;
  const bool zero = p.order == 1;
  const bool limit = p.limiter == FVH_LIMITER_BARTH_JESPERSEN;
#pragma omp parallel for schedule(static)
  for (int c0 = 0; c0 < m.num_cells; ++c0) {
    double u0[NV], u1[NV], umin[NV], umax[NV], phi[NV];
    double dudx[NV][D], grad_u[NV][D];
    double x0[D];
    for (int i = 0; i < D; ++i) x0[i] = m.cell_centroid[i][c0];
    if (zero) {
      for (int j = 0; j < NV; ++j)
        for (int i = 0; i < D; ++i) grad_u[j][i] = 0;
    } else {
      {
        int i = 0;
        u0[i++] = s.density[c0];
        for (int d = 0; d < D; ++d) u0[i++] = s.velocity[d][c0];
        u0[i++] = s.internal_energy[c0];
        u0[i++] = s.pressure[c0];
        u0[i++] = s.sound_speed[c0];
      }
      for (int i = 0; i < NV; ++i) umin[i] = umax[i] = u0[i];
      double dxdx[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int j = 0; j < NV; ++j)
        for (int i = 0; i < D; ++i) dudx[j][i] = 0;
      for (int q = m.cell_nbr_offsets[c0]; q < m.cell_nbr_offsets[c0 + 1]; ++q) {
        const int c1 = m.cell_nbrs[q];
        int i = 0;
        u1[i++] = s.density[c1];
        for (int d = 0; d < D; ++d) u1[i++] = s.velocity[d][c1];
        u1[i++] = s.internal_energy[c1];
        u1[i++] = s.pressure[c1];
        u1[i++] = s.sound_speed[c1];
        for (int k = 0; k < NV; ++k) {
          umin[k] = std::min(u1[k], umin[k]);
          umax[k] = std::max(u1[k], umax[k]);
        }
        double dx[D];
        for (int d = 0; d < D; ++d) dx[d] = m.cell_centroid[d][c1] - x0[d];
        if (D == 2) {
          dxdx[0][0] += dx[0] * dx[0];
          dxdx[0][1] += dx[0] * dx[1];
          dxdx[1][1] += dx[1] * dx[1];
        } else {
          dxdx[0][0] += dx[0] * dx[0];
          dxdx[0][1] += dx[0] * dx[1];
          dxdx[0][2] += dx[0] * dx[2];
          dxdx[1][1] += dx[1] * dx[1];
          dxdx[1][2] += dx[1] * dx[2];
          dxdx[2][2] += dx[2] * dx[2];
        }
        for (int k = 0; k < NV; ++k) {
          const double du = u1[k] - u0[k];
          for (int j = 0; j < D; ++j) dudx[k][j] += du * dx[j];
        }
      }
      if (D == 2) {
        const double denom =
            1 / (dxdx[0][0] * dxdx[1][1] - dxdx[0][1] * dxdx[0][1]);
        for (int j = 0; j < NV; ++j) {
          grad_u[j][0] = (dudx[j][0] * dxdx[1][1] - dudx[j][1] * dxdx[0][1]) * denom;
          grad_u[j][1] = (dudx[j][1] * dxdx[0][0] - dudx[j][0] * dxdx[0][1]) * denom;
        }
      } else {
        const double min1 = dxdx[1][1] * dxdx[2][2] - dxdx[1][2] * dxdx[1][2];
        const double min2 = dxdx[0][1] * dxdx[2][2] - dxdx[1][2] * dxdx[0][2];
        const double min3 = dxdx[0][1] * dxdx[1][2] - dxdx[1][1] * dxdx[0][2];
        const double denom =
            1 / (dxdx[0][0] * min1 - dxdx[0][1] * min2 + dxdx[0][2] * min3);
        for (int j = 0; j < NV; ++j) {
          const double *b = dudx[j];
          grad_u[j][0] = (b[0] * min1 - dxdx[0][1] * (b[1] * dxdx[2][2] - dxdx[1][2] * b[2]) +
                          dxdx[0][2] * (b[1] * dxdx[1][2] - dxdx[1][1] * b[2])) *
                         denom;
          grad_u[j][1] = (dxdx[0][0] * (b[1] * dxdx[2][2] - dxdx[1][2] * b[2]) - b[0] * min2 +
                          dxdx[0][2] * (b[2] * dxdx[0][1] - dxdx[0][2] * b[1])) *
                         denom;
          grad_u[j][2] = (dxdx[0][0] * (b[2] * dxdx[1][1] - dxdx[1][2] * b[1]) -
                          dxdx[0][1] * (b[2] * dxdx[0][1] - dxdx[0][2] * b[1]) + b[0] * min3) *
                         denom;
        }
      }
      if (limit) {
        for (int j = 0; j < NV; ++j) phi[j] = 1;
        for (int q = m.cell_vertex_offsets[c0]; q < m.cell_vertex_offsets[c0 + 1]; ++q) {
          const int vtx = m.cell_vertices[q];
          for (int j = 0; j < NV; ++j) u1[j] = u0[j];
          for (int i = 0; i < D; ++i) {
            const double dx = m.vertex_coord[i][vtx] - x0[i];
            for (int j = 0; j < NV; ++j) u1[j] += dx * grad_u[j][i];
          }
          for (int j = 0; j < NV; ++j) {
            const double du = u1[j] - u0[j];
            if (du > tol)
              phi[j] = std::min(phi[j], (umax[j] - u0[j]) / du);
            else if (du < -tol)
              phi[j] = std::min(phi[j], (umin[j] - u0[j]) / du);
          }
        }
        for (int j = 0; j < NV; ++j) {
          phi[j] = std::max<double>(phi[j], 0);
          for (int i = 0; i < D; ++i) grad_u[j][i] *= phi[j];
        }
      }
    }
    for (int i = 0; i < D; ++i) {
      int j = 0;
      g.density[i][c0] = grad_u[j++][i];
      for (int d = 0; d < D; ++d) g.velocity[d][i][c0] = grad_u[j++][i];
      g.internal_energy[i][c0] = grad_u[j++][i];
      g.pressure[i][c0] = grad_u[j++][i];
      g.sound_speed[i][c0] = grad_u[j++][i];
    }
  }
}

// pack_copy(c, d, v, p, e, T, a) + reconstruction at the face centroid
// (tasks.h:420-432).  With swap (the reference), the pressure slot receives the
// internal-energy gradient and the energy slot the pressure gradient.
template <int D>
inline prim<D> reconstruct(const fvh_mesh_view &m, const fvh_state_view &s,
                           const fvh_gradient_view &g, int c, int f, bool swap,
                           bool second) {
  prim<D> w;
  w.d = s.density[c];
  for (int i = 0; i < D; ++i) w.v[i] = s.velocity[i][c];
  w.p = s.pressure[c];
  w.e = s.internal_energy[c];
  w.T = s.temperature[c];
  w.a = s.sound_speed[c];
  if (!second) return w;
  double dx[D];
  for (int i = 0; i < D; ++i) dx[i] = m.face_centroid[i][f] - m.cell_centroid[i][c];
  const double *const *gp = swap ? g.internal_energy : g.pressure;
  const double *const *ge = swap ? g.pressure : g.internal_energy;
  for (int i = 0; i < D; ++i) {
    w.d += dx[i] * g.density[i][c];
    for (int d = 0; d < D; ++d) w.v[d] += dx[i] * g.velocity[d][i][c];
    w.p += dx[i] * gp[i][c];
    w.e += dx[i] * ge[i][c];
    w.a += dx[i] * g.sound_speed[i][c];
  }
  return w;
}

template <int D>
void evaluate_fluxes(const fvh_mesh_view &m, const fvh_state_view &s,
                     const fvh_gradient_view &g, const fvh_flux_view &fl,
                     const fvh_params &p) {
  const bool swap = p.recon_swap_ep != 0;
  const bool second = p.order != 1;
#pragma omp parallel for schedule(static)
  for (int f = 0; f < m.num_faces; ++f) {
    const int c0 = m.face_cells[2 * (size_t)f];
    const int c1 = m.face_cells[2 * (size_t)f + 1];
    double n[D];
    for (int i = 0; i < D; ++i) n[i] = m.face_normal[i][f];
    const prim<D> wl = reconstruct<D>(m, s, g, c0, f, swap, second);
    double F[D + 2];
    if (c1 >= 0) {
      const prim<D> wr = reconstruct<D>(m, s, g, c1, f, swap, second);
      if (p.flux_kind == FVH_FLUX_RUSANOV)
        rusanov<D>(wl, wr, n, F);
      else if (p.flux_kind == FVH_FLUX_HLLC)
        hllc<D>(wl, wr, n, F);
      else
        hlle<D>(wl, wr, n, F);
    } else if (p.boundary == FVH_BOUNDARY_OUTFLOW) {
      phys_flux<D>(wl, n, F);  // transmissive: ghost state = interior state
    } else {
      wall<D>(wl, n, F);
    }
    const double area = m.face_area[f];
    fl.mass[f] = F[0] * area;
    for (int i = 0; i < D; ++i) fl.momentum[i][f] = F[1 + i] * area;
    fl.energy[f] = F[D + 1] * area;
  }
}

// update_state_from_flux (euler_eqns.h:383-410) then update_state_from_energy
// (euler_eqns.h:359-375) with ideal_gas_t (ideal_gas.h:193-226) on one cell;
// w = (d, v[D], p, e, T, a), du already scaled by delta_t / V.
template <int D>
inline void update_cell(double gamma, double cv, double *w, const double *du) {
  double vel[D];
  for (int i = 0; i < D; ++i) vel[i] = w[1 + i];
  const double den0 = w[0];
  const double mass = den0 + du[0];
  const double ener = den0 * (w[D + 2] + 0.5 * dot<D>(vel, vel)) + du[D + 1];
  const double inv_mass = 1 / mass;
  for (int i = 0; i < D; ++i) {
    const double mom = den0 * vel[i] + du[1 + i];
    vel[i] = mom * inv_mass;
  }
  const double e = ener * inv_mass - 0.5 * dot<D>(vel, vel);
  w[0] = mass;
  for (int i = 0; i < D; ++i) w[1 + i] = vel[i];
  w[D + 2] = e;
  w[D + 1] = (gamma - 1.0) * mass * e;
  w[D + 3] = e / cv;
  w[D + 4] = std::sqrt(gamma * (gamma - 1.0) * e);
}

template <int D>
int apply_update(const fvh_mesh_view &m, const fvh_params &p, double dt,
                 double factor, const fvh_flux_view &fl, const fvh_state_view &s,
                 double *soln_time, int64_t *bad_cell) {
  double delta_t = dt;
  delta_t *= factor;
  *soln_time = 0.0 + *soln_time + delta_t;  // initial_soln_time + old + delta_t
  int64_t first_bad = INT64_MAX;
#pragma omp parallel for schedule(static) reduction(min : first_bad)
  for (int c = 0; c < m.num_cells; ++c) {
    double du[D + 2];
    for (int k = 0; k < D + 2; ++k) du[k] = 0;
    for (int q = m.cell_face_offsets[c]; q < m.cell_face_offsets[c + 1]; ++q) {
      const int sf = m.cell_faces[q];
      const int f = sf < 0 ? ~sf : sf;
      double F[D + 2];
      F[0] = fl.mass[f];
      for (int i = 0; i < D; ++i) F[1 + i] = fl.momentum[i][f];
      F[D + 1] = fl.energy[f];
      if (sf >= 0)
        for (int k = 0; k < D + 2; ++k) du[k] -= F[k];
      else
        for (int k = 0; k < D + 2; ++k) du[k] += F[k];
    }
    const double scale = delta_t / m.cell_volume[c];
    for (int k = 0; k < D + 2; ++k) du[k] *= scale;
    double w[D + 5];
    w[0] = s.density[c];
    for (int i = 0; i < D; ++i) w[1 + i] = s.velocity[i][c];
    w[D + 1] = s.pressure[c];
    w[D + 2] = s.internal_energy[c];
    w[D + 3] = s.temperature[c];
    w[D + 4] = s.sound_speed[c];
    update_cell<D>(p.gamma, p.cv, w, du);
    const double mass = w[0], e = w[D + 2];
    s.density[c] = mass;
    for (int i = 0; i < D; ++i) s.velocity[i][c] = w[1 + i];
    s.internal_energy[c] = e;
    s.pressure[c] = w[D + 1];
    s.temperature[c] = w[D + 3];
    s.sound_speed[c] = w[D + 4];
    if (e < 0 || mass < 0) first_bad = std::min<int64_t>(first_bad, c);
  }
  if (first_bad != INT64_MAX) {
    if (bad_cell) *bad_cell = first_bad;
    return FVH_ERR_NEGATIVE_STATE;
  }
  return FVH_OK;
}

struct work {
  std::vector<double> buf;
  fvh_gradient_view g;
  fvh_flux_view f;
  work(int dim, int nc, int nf) {
    const int ng = (dim + 4) * dim;
    buf.assign((size_t)ng * nc + (size_t)(dim + 2) * nf, 0.0);
    std::memset(&g, 0, sizeof g);
    std::memset(&f, 0, sizeof f);
    double *b = buf.data();
    auto take = [&](size_t n) {
      double *r = b;
      b += n;
      return r;
    };
    for (int i = 0; i < dim; ++i) g.density[i] = take(nc);
    for (int d = 0; d < dim; ++d)
      for (int i = 0; i < dim; ++i) g.velocity[d][i] = take(nc);
    for (int i = 0; i < dim; ++i) g.internal_energy[i] = take(nc);
    for (int i = 0; i < dim; ++i) g.pressure[i] = take(nc);
    for (int i = 0; i < dim; ++i) g.sound_speed[i] = take(nc);
    f.mass = take(nf);
    for (int i = 0; i < dim; ++i) f.momentum[i] = take(nf);
    f.energy = take(nf);
  }
};

template <int D>
int run(const fvh_mesh_view &m, const fvh_params &p, const fvh_state_view &s,
        int64_t nsteps, int stop_at_final, double *soln_time, int64_t *steps_done,
        int64_t *bad_cell) {
  work w(D, m.num_cells, m.num_faces);
  int64_t n = 0;
  int st = FVH_OK;
  for (; n < nsteps; ++n) {
    if (stop_at_final && *soln_time >= p.final_time - 1e-12 * std::abs(p.final_time))
      break;
    const double dt = evaluate_time_step<D>(m, s, p, *soln_time, &st);
    if (st != FVH_OK) break;
    for (int stage = 0; stage < 2; ++stage) {
      evaluate_gradients<D>(m, s, w.g, p);
      evaluate_fluxes<D>(m, s, w.g, w.f, p);
      st = apply_update<D>(m, p, dt, 0.5, w.f, s, soln_time, bad_cell);
      if (st != FVH_OK) break;
    }
    if (st != FVH_OK) {
      ++n;
      break;
    }
  }
  if (steps_done) *steps_done = n;
  return st;
}

}  // namespace

extern "C" {

int oracle_evaluate_time_step(const fvh_mesh_view *m, const fvh_state_view *s,
                              const fvh_params *p, double soln_time, double *dt) {
  int st = FVH_OK;
  *dt = m->dim == 2 ? evaluate_time_step<2>(*m, *s, *p, soln_time, &st)
                    : evaluate_time_step<3>(*m, *s, *p, soln_time, &st);
  return st;
}

void oracle_evaluate_gradients(const fvh_mesh_view *m, const fvh_state_view *s,
                               const fvh_gradient_view *g, const fvh_params *p) {
  if (m->dim == 2)
    evaluate_gradients<2>(*m, *s, *g, *p);
  else
    evaluate_gradients<3>(*m, *s, *g, *p);
}

void oracle_evaluate_fluxes(const fvh_mesh_view *m, const fvh_state_view *s,
                            const fvh_gradient_view *g, const fvh_flux_view *f,
                            const fvh_params *p) {
  if (m->dim == 2)
    evaluate_fluxes<2>(*m, *s, *g, *f, *p);
  else
    evaluate_fluxes<3>(*m, *s, *g, *f, *p);
}

int oracle_apply_update(const fvh_mesh_view *m, const fvh_params *p, double dt,
                        double factor, const fvh_flux_view *f,
                        const fvh_state_view *s, double *soln_time,
                        int64_t *bad_cell) {
  return m->dim == 2 ? apply_update<2>(*m, *p, dt, factor, *f, *s, soln_time, bad_cell)
                     : apply_update<3>(*m, *p, dt, factor, *f, *s, soln_time, bad_cell);
}

int oracle_run(const fvh_mesh_view *m, const fvh_params *p, const fvh_state_view *s,
               int64_t nsteps, int stop_at_final, double *soln_time,
               int64_t *steps_done, int64_t *bad_cell) {
  return m->dim == 2 ? run<2>(*m, *p, *s, nsteps, stop_at_final, soln_time, steps_done, bad_cell)
                     : run<3>(*m, *p, *s, nsteps, stop_at_final, soln_time, steps_done, bad_cell);
}

// update_state_from_pressure (euler_eqns.h:333-350) with ideal_gas_t
// (ideal_gas.h:178-226): e, T, a from d, p.
void oracle_state_from_pressure(int32_t n, double gamma, double cv,
                                const double *d, const double *p, double *e,
                                double *T, double *a) {
  for (int32_t i = 0; i < n; ++i) {
    const double ie = p[i] / (d[i] * (gamma - 1.0));
    e[i] = ie;
    T[i] = ie / cv;
    a[i] = std::sqrt(gamma * (gamma - 1.0) * ie);
  }
}

void oracle_update_cell(int32_t dim, double gamma, double cv, double *w, const double *du) {
  if (dim == 2)
    update_cell<2>(gamma, cv, w, du);
  else
    update_cell<3>(gamma, cv, w, du);
}

// Single-face flux functions for unit checks: w = (d, v[dim], p, e, T, a).
void oracle_face_flux(int32_t dim, int32_t kind, const double *wl,
                      const double *wr, const double *n, double *f) {
  auto load2 = [](const double *w) {
    prim<2> u;
    u.d = w[0]; u.v[0] = w[1]; u.v[1] = w[2]; u.p = w[3]; u.e = w[4]; u.T = w[5]; u.a = w[6];
    return u;
  };
  auto load3 = [](const double *w) {
    prim<3> u;
    u.d = w[0]; u.v[0] = w[1]; u.v[1] = w[2]; u.v[2] = w[3]; u.p = w[4]; u.e = w[5]; u.T = w[6]; u.a = w[7];
    return u;
  };
  if (dim == 2) {
    const prim<2> l = load2(wl);
    if (kind < 0) { wall<2>(l, n, f); return; }
    const prim<2> r = load2(wr);
    if (kind == FVH_FLUX_RUSANOV) rusanov<2>(l, r, n, f);
    else if (kind == FVH_FLUX_HLLC) hllc<2>(l, r, n, f);
    else hlle<2>(l, r, n, f);
  } else {
    const prim<3> l = load3(wl);
    if (kind < 0) { wall<3>(l, n, f); return; }
    const prim<3> r = load3(wr);
    if (kind == FVH_FLUX_RUSANOV) rusanov<3>(l, r, n, f);
    else if (kind == FVH_FLUX_HLLC) hllc<3>(l, r, n, f);
    else hlle<3>(l, r, n, f);
  }
}

// OpenMP threads the oracle's loops use (the CPU baseline times 1 and all).
void oracle_set_threads(int32_t n) { omp_set_num_threads(n > 0 ? n : omp_get_num_procs()); }
int32_t oracle_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
