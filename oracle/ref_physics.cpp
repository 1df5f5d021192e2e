// Compiles the reference's own physics headers (flecsale/eqns/euler_eqns.h,
// flecsale/eqns/flux.h, flecsale/eos/ideal_gas.h, included unchanged from the
// reference checkout) behind a C interface, so the oracle's restatement can be
// compared with the reference's code bit for bit.  Test infrastructure only;
// built into oracle/_ref by ref_build.py.
#include <cstdint>
#include <tuple>

#include <flecsale/eos/ideal_gas.h>
#include <flecsale/eqns/euler_eqns.h>
#include <flecsale/eqns/flux.h>

namespace {

template <int D>
using eqns = flecsale::eqns::euler_eqns_t<double, D>;
template <int D>
using vec = ristra::math::array<double, D>;

// w = (d, v[D], p, e, T, a) -> pack_copy tuple (apps/hydro/types.h:150-155)
template <int D>
auto load(const double *w) {
  vec<D> v;
  for (int i = 0; i < D; ++i) v[i] = w[1 + i];
  return std::make_tuple(w[0], v, w[D + 1], w[D + 2], w[D + 3], w[D + 4]);
}

template <int D>
void flux(int kind, const double *wl, const double *wr, const double *n, double *f) {
  vec<D> nn;
  for (int i = 0; i < D; ++i) nn[i] = n[i];
  auto l = load<D>(wl);
  typename eqns<D>::flux_data_t r;
  if (kind < 0) {
    r = eqns<D>::wall_flux(l, nn);
  } else {
    auto rr = load<D>(wr);
    if (kind == 1)
      r = flecsale::eqns::rusanov_flux<eqns<D>>(l, rr, nn);
    else
      r = flecsale::eqns::hlle_flux<eqns<D>>(l, rr, nn);
  }
  for (int i = 0; i < D + 2; ++i) f[i] = r[i];
}

// apply_update's per-cell work (tasks.h:646-651) on one cell: w in/out.
template <int D>
void update(double gamma, double cv, double *w, const double *du_in) {
  double d = w[0], p = w[D + 1], e = w[D + 2], T = w[D + 3], a = w[D + 4];
  vec<D> v;
  for (int i = 0; i < D; ++i) v[i] = w[1 + i];
  typename eqns<D>::flux_data_t du;
  for (int i = 0; i < D + 2; ++i) du[i] = du_in[i];
  auto u = std::forward_as_tuple(d, v, p, e, T, a);
  flecsale::eos::ideal_gas_t<double> eos(gamma, cv);
  eqns<D>::update_state_from_flux(u, du);
  eqns<D>::update_state_from_energy(u, eos);
  w[0] = d;
  for (int i = 0; i < D; ++i) w[1 + i] = v[i];
  w[D + 1] = p;
  w[D + 2] = e;
  w[D + 3] = T;
  w[D + 4] = a;
}

}  // namespace

extern "C" {

void ref_face_flux(int32_t dim, int32_t kind, const double *wl, const double *wr,
                   const double *n, double *f) {
  if (dim == 2)
    flux<2>(kind, wl, wr, n, f);
  else
    flux<3>(kind, wl, wr, n, f);
}

void ref_update_cell(int32_t dim, double gamma, double cv, double *w, const double *du) {
  if (dim == 2)
    update<2>(gamma, cv, w, du);
  else
    update<3>(gamma, cv, w, du);
}

// update_state_from_pressure (euler_eqns.h:333-350)
void ref_state_from_pressure(double gamma, double cv, double d, double p, double *e,
                             double *T, double *a) {
  double dd = d, pp = p, ee = 0, TT = 0, aa = 0;
  ristra::math::array<double, 2> v(0.0);
  auto u = std::forward_as_tuple(dd, v, pp, ee, TT, aa);
  flecsale::eos::ideal_gas_t<double> eos(gamma, cv);
  eqns<2>::update_state_from_pressure(u, eos);
  *e = ee;
  *T = TT;
  *a = aa;
}

}  // extern "C"
