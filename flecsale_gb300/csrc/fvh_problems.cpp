// Initial conditions (apps/hydro/tasks.h:46-68): per cell (density, velocity,
// pressure) from the cell centroid, then the EOS closure of
// update_state_from_pressure (flecsale/eqns/euler_eqns.h:333-350) with the
// ideal gas of flecsale/eos/ideal_gas.h:178-226.
#include <cmath>

#include "flecsale_gb300.h"
#include "fvh_internal.h"

namespace {

struct dvp {
  double d, v[3], p;
};

dvp problem_state(int kind, int dim, const double *x, int64_t cell, uint64_t seed) {
  dvp s{1.0, {0, 0, 0}, 1.0};
  switch (kind) {
    case FVH_PROBLEM_SHOCK_BOX: {  // apps/hydro/2d/inputs.cc:51-58, 3d/inputs.cc:127-134
      bool low = true;
      for (int k = 0; k < dim; ++k) low = low && x[k] < 0;
      if (low) {
        s.d = 0.125;
        s.p = 0.1;
      }
      break;
    }
    case FVH_PROBLEM_SOD:
      if (!(x[0] < 0.5)) {
        s.d = 0.125;
        s.p = 0.1;
      }
      break;
    case FVH_PROBLEM_FOUR_QUADRANT: {
      const bool east = x[0] >= 0.5, north = x[1] >= 0.5;
      if (east && north) {
        s.d = 1.5; s.p = 1.5;
      } else if (!east && north) {
        s.d = 0.5323; s.v[0] = 1.206; s.p = 0.3;
      } else if (!east && !north) {
        s.d = 0.138; s.v[0] = 1.206; s.v[1] = 1.206; s.p = 0.029;
      } else {
        s.d = 0.5323; s.v[1] = 1.206; s.p = 0.3;
      }
      break;
    }
    case FVH_PROBLEM_INNER_CUBE: {
      bool in = true;
      for (int k = 0; k < dim; ++k) in = in && x[k] < 0.5;
      if (!in) {
        s.d = 0.125;
        s.p = 0.1;
      }
      break;
    }
    case FVH_PROBLEM_KELVIN_HELMHOLTZ: {
      const bool strip = std::fabs(x[1] - 0.5) < 0.25;
      s.d = strip ? 2.0 : 1.0;
      s.v[0] = strip ? 0.5 : -0.5;
      const double noise = 2.0 * fvh::uniform01(seed, (uint64_t)cell) - 1.0;
      s.v[1] = 0.01 * std::sin(4.0 * M_PI * x[0]) + 1e-3 * noise;
      s.p = 2.5;
      break;
    }
    default:  // FVH_PROBLEM_UNIFORM
      break;
  }
  return s;
}

}  // namespace

extern "C" {

fvh_status fvh_host_initial_state(int32_t kind, const fvh_host_mesh *m,
                                  const fvh_params *p, uint64_t seed,
                                  double *host_planes) {
  if (!m || !p || !host_planes || kind < 0 || kind > FVH_PROBLEM_UNIFORM ||
      p->dim != m->dim || !(p->gamma > 1) || !(p->cv > 0))
    return FVH_ERR_INVALID_ARGUMENT;
  const int dim = m->dim;
  const int64_t nc = m->nc;
  double *d = host_planes;
  double *v[3] = {host_planes + nc, host_planes + 2 * nc, host_planes + 3 * nc};
  double *e = host_planes + (1 + dim) * nc;
  double *pr = e + nc, *T = pr + nc, *a = T + nc;
  const double gamma = p->gamma, cv = p->cv;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    double x[3] = {0, 0, 0};
    for (int k = 0; k < dim; ++k) x[k] = m->cc[k][c];
    const dvp s = problem_state(kind, dim, x, c, seed);
    d[c] = s.d;
    for (int k = 0; k < dim; ++k) v[k][c] = s.v[k];
    pr[c] = s.p;
    const double ie = s.p / (s.d * (gamma - 1.0));
    e[c] = ie;
    T[c] = ie / cv;
    a[c] = std::sqrt(gamma * (gamma - 1.0) * ie);
  }
  return FVH_OK;
}

}  // extern "C"
