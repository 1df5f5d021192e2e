// Euler flux physics on one face, templated on the scalar type.
//
// T = double (compiled without FMA contraction) reproduces the reference's
// rounding; T = float is the mixed-precision form's flux arithmetic.  The
// statement order follows
//   euler_eqns_t::total_energy     flecsale/eqns/euler_eqns.h:167-173
//   euler_eqns_t::flux             flecsale/eqns/euler_eqns.h:274-304
//   euler_eqns_t::solution_delta   flecsale/eqns/euler_eqns.h:238-265
//   minmax_eigenvalues             flecsale/eqns/euler_eqns.h:222-230
//   fastest_wavespeed              flecsale/eqns/euler_eqns.h:183-189
//   hlle_flux                      flecsale/eqns/flux.h:79-106
//   rusanov_flux                   flecsale/eqns/flux.h:51-65
//   wall_flux                      flecsale/eqns/euler_eqns.h:313-324
// with ristra's dot_product summing from zero in index order.  HLLC (not in the
// reference) follows Toro, "Riemann Solvers and Numerical Methods for Fluid
// Dynamics", sec. 10.4, with the HLLE wave-speed estimates.
#pragma once

#include "flecsale_gb300.h"

namespace fvh {
namespace phys {

// std::max / std::min semantics (a < b ? b : a)
template <typename T>
__device__ __forceinline__ T smax(T a, T b) { return (a < b) ? b : a; }
template <typename T>
__device__ __forceinline__ T smin(T a, T b) { return (b < a) ? b : a; }

template <typename T, int D>
__device__ __forceinline__ T dot(const T *a, const T *b) {
  T s = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) s += a[i] * b[i];
  return s;
}

// Slots of pack_copy(c, d, v, p, e, T, a) (apps/hydro/tasks.h:420); the
// temperature slot is never read by a flux and is left out.
template <typename T, int D>
struct prim {
  T d, v[D], p, e, a;
};

template <typename T, int D>
__device__ __forceinline__ T total_energy(const prim<T, D> &u) {
  return u.e + T(0.5) * dot<T, D>(u.v, u.v);
}

template <typename T, int D>
__device__ __forceinline__ void phys_flux(const prim<T, D> &u, const T *n, T *f) {
  const T et = total_energy<T, D>(u);
  const T vn = dot<T, D>(u.v, n);
  const T mass_flux = u.d * vn;
  f[0] = mass_flux;
#pragma unroll
  for (int i = 0; i < D; ++i) f[1 + i] = mass_flux * u.v[i] + u.p * n[i];
  f[D + 1] = mass_flux * (et + u.p / u.d);
}

template <typename T, int D>
__device__ __forceinline__ void solution_delta(const prim<T, D> &l, const prim<T, D> &r, T *du) {
  const T ener_l = l.d * total_energy<T, D>(l);
  const T ener_r = r.d * total_energy<T, D>(r);
  du[0] = r.d - l.d;
#pragma unroll
  for (int i = 0; i < D; ++i) du[1 + i] = r.d * r.v[i] - l.d * l.v[i];
  du[D + 1] = ener_r - ener_l;
}

template <typename T, int D>
__device__ __forceinline__ void hlle(const prim<T, D> &l, const prim<T, D> &r, const T *n, T *f) {
  const T vnl = dot<T, D>(l.v, n), vnr = dot<T, D>(r.v, n);
  const T lambda_l = smin(vnl - l.a, vnr - r.a);
  const T lambda_r = smax(vnl + l.a, vnr + r.a);
  if (lambda_l >= 0) {
    phys_flux<T, D>(l, n, f);
  } else if (lambda_r <= 0) {
    phys_flux<T, D>(r, n, f);
  } else {
    T fl[D + 2], fr[D + 2], du[D + 2];
    phys_flux<T, D>(l, n, fl);
    phys_flux<T, D>(r, n, fr);
    const T c1 = lambda_l * lambda_r;
    const T c2 = lambda_r - lambda_l;
    const T c2inv = T(1) / c2;
    solution_delta<T, D>(l, r, du);
#pragma unroll
    for (int i = 0; i < D + 2; ++i) f[i] = c2inv * (lambda_r * fl[i] - lambda_l * fr[i] + c1 * du[i]);
  }
}

template <typename T, int D>
__device__ __forceinline__ void rusanov(const prim<T, D> &l, const prim<T, D> &r, const T *n, T *f) {
  T fl[D + 2], fr[D + 2], du[D + 2];
  phys_flux<T, D>(l, n, fl);
  phys_flux<T, D>(r, n, fr);
  const T sl = l.a + fabs(dot<T, D>(l.v, n));
  const T sr = r.a + fabs(dot<T, D>(r.v, n));
  const T s = smax(sl, sr);
  solution_delta<T, D>(l, r, du);
  const T half_s = s / T(2);
#pragma unroll
  for (int i = 0; i < D + 2; ++i) f[i] = (fl[i] + fr[i]) / T(2) - du[i] * half_s;
}

template <typename T, int D>
__device__ __forceinline__ void hllc(const prim<T, D> &l, const prim<T, D> &r, const T *n, T *f) {
  const T vnl = dot<T, D>(l.v, n), vnr = dot<T, D>(r.v, n);
  const T sL = smin(vnl - l.a, vnr - r.a);
  const T sR = smax(vnl + l.a, vnr + r.a);
  if (sL >= 0) {
    phys_flux<T, D>(l, n, f);
    return;
  }
  if (sR <= 0) {
    phys_flux<T, D>(r, n, f);
    return;
  }
  const T ml = l.d * (sL - vnl);
  const T mr = r.d * (sR - vnr);
  const T sM = (r.p - l.p + ml * vnl - mr * vnr) / (ml - mr);
  const bool left = sM >= 0;
  const prim<T, D> &u = left ? l : r;
  const T sK = left ? sL : sR;
  const T mK = left ? ml : mr;
  const T vnK = left ? vnl : vnr;
  T fk[D + 2];
  phys_flux<T, D>(u, n, fk);
  const T EK = u.d * total_energy<T, D>(u);
  const T fac = mK / (sK - sM);
  const T dvn = sM - vnK;
  f[0] = fk[0] + sK * (fac - u.d);
#pragma unroll
  for (int i = 0; i < D; ++i) f[1 + i] = fk[1 + i] + sK * (fac * (u.v[i] + dvn * n[i]) - u.d * u.v[i]);
  f[D + 1] = fk[D + 1] + sK * (fac * (EK / u.d + dvn * (sM + u.p / mK)) - EK);
}

template <typename T, int D>
__device__ __forceinline__ void wall(const prim<T, D> &u, const T *n, T *f) {
  f[0] = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) f[1 + i] = u.p * n[i];
  f[D + 1] = 0;
}

template <typename T, int D, int KIND>
__device__ __forceinline__ void riemann(const prim<T, D> &l, const prim<T, D> &r, const T *n, T *f) {
  if (KIND == FVH_FLUX_RUSANOV)
    rusanov<T, D>(l, r, n, f);
  else if (KIND == FVH_FLUX_HLLC)
    hllc<T, D>(l, r, n, f);
  else
    hlle<T, D>(l, r, n, f);
}

}  // namespace phys
}  // namespace fvh
