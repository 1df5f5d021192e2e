// C ABI of the hydro step: argument checking, the task entry points, the solver
// object (work buffers + the time loop of apps/hydro/driver.h:317-413) and the
// device-memory helpers.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "flecsale_gb300.h"
#include "fvh_internal.h"
#include "fvh_kernels.h"
#include "fvh_checks.h"
#include "fvh_mixed.h"

namespace {

using fvh::from_cuda;
using fvh::mesh_ok;
using fvh::state_ok;
using fvh::grads_ok;
using fvh::flux_ok;
using fvh::params_ok;

inline cudaStream_t cs(fvh_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

int dt_blocks(int num_cells) {
  int nb = (num_cells + fvh::kDtThreads - 1) / fvh::kDtThreads;
  return nb < fvh::kDtMaxBlocks ? nb : fvh::kDtMaxBlocks;
}

}  // namespace

// ---------------------------------------------------------------------------
// solver object
// ---------------------------------------------------------------------------
struct fvh_solver {
  fvh_mesh_view mesh{};
  fvh_params params{};
  fvh_gradient_view grads{};
  fvh_flux_view flux{};
  double *work = nullptr;          // gradients + fluxes
  double *tables = nullptr;        // FP64 path: geometry-only tables (one allocation)
  fvh::plain::tables tab;          // views into `tables`
  double *scalars = nullptr;       // [0] soln time, [1] dt, [2..] dt partials
  fvh_device_status *status = nullptr;
  double *host_scalars = nullptr;  // pinned: soln time
  fvh_device_status *host_status = nullptr;
  fvh::mixed::workspace *mixed = nullptr;
  fvh::mixed::launch_shape shape;  // mixed form's cell-kernel launch shape
  // one CUDA graph per step variant (index: pack_first * 2 + write_next), for
  // one (stream, state) pair
  cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaStream_t graph_stream = nullptr;
  fvh_state_view graph_state{};
};

static void drop_graphs(fvh_solver *s) {
  for (auto &g : s->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}


struct fvh_device_state {
  fvh_state_view view{};
  double *base = nullptr;
};

extern "C" {

const char *fvh_status_string(int32_t s) {
  switch (s) {
    case FVH_OK: return "ok";
    case FVH_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FVH_ERR_CUDA: return "CUDA runtime error";
    case FVH_ERR_INFINITE_DT: return "infinite delta t";
    case FVH_ERR_NEGATIVE_STATE: return "Negative density or internal energy encountered!";
    case FVH_ERR_UNSUPPORTED: return "unsupported mesh or option";
    case FVH_ERR_NO_DEVICE: return "no CUDA device";
    case FVH_ERR_OUT_OF_MEMORY: return "out of device memory";
    case FVH_ERR_CAPACITY: return "request exceeds a fixed capacity";
    case FVH_ERR_TIMEOUT: return "a kernel's bounded wait on its data copies ran out";
    default: return "unknown status";
  }
}

int32_t fvh_abi_version(void) { return FVH_ABI_VERSION; }

void fvh_params_default(fvh_params *p, int32_t dim) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->dim = dim;
  p->flux_kind = FVH_FLUX_HLLE;
  p->limiter = FVH_LIMITER_BARTH_JESPERSEN;
  p->order = 2;
  p->recon_swap_ep = 1;
  p->precision = FVH_PRECISION_FP64;
  p->gamma = 1.4;
  p->cv = 1.0;
  p->cfl = dim == 3 ? 1.0 / 3.0 : 0.5;
  p->final_time = 0.2;
}

void fvh_status_decode(fvh_device_status s, int32_t *code, int64_t *cell) {
  if (s == FVH_STATUS_CLEAR) {
    if (code) *code = FVH_OK;
    if (cell) *cell = -1;
    return;
  }
  if (code) *code = (int32_t)(s & 0xff);
  if (cell) *cell = (int64_t)(s >> 8);
}

size_t fvh_time_step_workspace_bytes(int32_t num_cells) {
  return sizeof(double) * (size_t)dt_blocks(num_cells > 0 ? num_cells : 1);
}

fvh_status fvh_evaluate_time_step(const fvh_mesh_view *mesh, const fvh_state_view *state,
                                  const fvh_params *params, const double *d_soln_time,
                                  double *d_dt, void *d_workspace, size_t workspace_bytes,
                                  fvh_device_status *d_status, fvh_stream_t stream) {
  if (!mesh_ok(mesh) || !state_ok(state, mesh->dim) || !params_ok(params, mesh->dim) ||
      !d_soln_time || !d_dt || !d_workspace || !d_status ||
      workspace_bytes < fvh_time_step_workspace_bytes(mesh->num_cells))
    return FVH_ERR_INVALID_ARGUMENT;
  const int nb = dt_blocks(mesh->num_cells);
  double *partial = static_cast<double *>(d_workspace);
  const cudaError_t e =
      mesh->dim == 2
          ? fvh::plain::launch_dt<2>(*mesh, *state, *params, d_soln_time, d_dt, partial, nb,
                                     d_status, cs(stream))
          : fvh::plain::launch_dt<3>(*mesh, *state, *params, d_soln_time, d_dt, partial, nb,
                                     d_status, cs(stream));
  return from_cuda(e);
}

fvh_status fvh_evaluate_gradients(const fvh_mesh_view *mesh, const fvh_state_view *state,
                                  const fvh_gradient_view *grads, const fvh_params *params,
                                  fvh_stream_t stream) {
  if (!mesh_ok(mesh) || !state_ok(state, mesh->dim) || !grads_ok(grads, mesh->dim) ||
      !params_ok(params, mesh->dim))
    return FVH_ERR_INVALID_ARGUMENT;
  if (params->order == 1) {
    // first order: zero gradients
    const int D = mesh->dim;
    for (int i = 0; i < D; ++i) {
      const size_t b = sizeof(double) * mesh->num_cells;
      cudaMemsetAsync(grads->density[i], 0, b, cs(stream));
      cudaMemsetAsync(grads->internal_energy[i], 0, b, cs(stream));
      cudaMemsetAsync(grads->pressure[i], 0, b, cs(stream));
      cudaMemsetAsync(grads->sound_speed[i], 0, b, cs(stream));
      for (int d = 0; d < D; ++d) cudaMemsetAsync(grads->velocity[d][i], 0, b, cs(stream));
    }
    return from_cuda(cudaGetLastError());
  }
  const cudaError_t e =
      mesh->dim == 2 ? fvh::plain::launch_gradients<2>(*mesh, *state, *grads, *params, cs(stream))
                     : fvh::plain::launch_gradients<3>(*mesh, *state, *grads, *params, cs(stream));
  return from_cuda(e);
}

fvh_status fvh_evaluate_fluxes(const fvh_mesh_view *mesh, const fvh_state_view *state,
                               const fvh_gradient_view *grads, const fvh_flux_view *flux,
                               const fvh_params *params, fvh_stream_t stream) {
  if (!mesh_ok(mesh) || !state_ok(state, mesh->dim) || !grads_ok(grads, mesh->dim) ||
      !flux_ok(flux, mesh->dim) || !params_ok(params, mesh->dim))
    return FVH_ERR_INVALID_ARGUMENT;
  const cudaError_t e =
      mesh->dim == 2
          ? fvh::plain::launch_fluxes<2>(*mesh, *state, *grads, *flux, *params, cs(stream))
          : fvh::plain::launch_fluxes<3>(*mesh, *state, *grads, *flux, *params, cs(stream));
  return from_cuda(e);
}

fvh_status fvh_apply_update(const fvh_mesh_view *mesh, const fvh_params *params,
                            const double *d_dt, double factor, const fvh_flux_view *flux,
                            const fvh_state_view *state, double *d_soln_time,
                            fvh_device_status *d_status, fvh_stream_t stream) {
  if (!mesh_ok(mesh) || !state_ok(state, mesh->dim) || !flux_ok(flux, mesh->dim) ||
      !params_ok(params, mesh->dim) || !d_dt || !d_soln_time || !d_status)
    return FVH_ERR_INVALID_ARGUMENT;
  const cudaError_t e =
      mesh->dim == 2 ? fvh::plain::launch_update<2>(*mesh, *params, d_dt, factor, *flux, *state,
                                                    d_soln_time, d_status, cs(stream))
                     : fvh::plain::launch_update<3>(*mesh, *params, d_dt, factor, *flux, *state,
                                                    d_soln_time, d_status, cs(stream));
  return from_cuda(e);
}

// ---------------------------------------------------------------------------
// solver
// ---------------------------------------------------------------------------
void fvh_solver_destroy(fvh_solver *s) {
  if (!s) return;
  drop_graphs(s);
  if (s->mixed) fvh::mixed::destroy(s->mixed);
  cudaFree(s->work);
  cudaFree(s->tables);
  cudaFree(s->scalars);
  cudaFree(s->status);
  cudaFreeHost(s->host_scalars);
  cudaFreeHost(s->host_status);
  delete s;
}

fvh_status fvh_solver_create(const fvh_mesh_view *mesh, const fvh_params *params,
                             fvh_solver **out) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!out || !mesh_ok(mesh) || !params_ok(params, mesh->dim)) return FVH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    fvh_solver *s = new (std::nothrow) fvh_solver();
    if (!s) return FVH_ERR_OUT_OF_MEMORY;
    s->mesh = *mesh;
    s->params = *params;
    const int D = mesh->dim;
    const size_t nc = mesh->num_cells, nf = mesh->num_faces;
    const size_t ng = (size_t)(D + 4) * D;
    cudaError_t e = cudaSuccess;
    if (params->precision == FVH_PRECISION_FP64) {
      e = cudaMalloc(&s->work, sizeof(double) * (ng * nc + (size_t)(D + 2) * nf));
      if (e == cudaSuccess) {
        double *b = s->work;
        for (int i = 0; i < D; ++i, b += nc) s->grads.density[i] = b;
        for (int d = 0; d < D; ++d)
          for (int i = 0; i < D; ++i, b += nc) s->grads.velocity[d][i] = b;
        for (int i = 0; i < D; ++i, b += nc) s->grads.internal_energy[i] = b;
        for (int i = 0; i < D; ++i, b += nc) s->grads.pressure[i] = b;
        for (int i = 0; i < D; ++i, b += nc) s->grads.sound_speed[i] = b;
        s->flux.mass = b;
        b += nf;
        for (int i = 0; i < D; ++i, b += nf) s->flux.momentum[i] = b;
        s->flux.energy = b;
      }
      // geometry-only tables (built once, same arithmetic as on the fly)
      int32_t nnz[3] = {0, 0, 0};
      const int32_t *offs[3] = {mesh->cell_face_offsets, mesh->cell_nbr_offsets,
                                mesh->cell_vertex_offsets};
      for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        e = cudaMemcpy(&nnz[k], offs[k] + nc, sizeof(int32_t), cudaMemcpyDeviceToHost);
      const size_t ntab = fvh::plain::table_doubles(D, nc, nf, nnz[0], nnz[1], nnz[2]);
      if (e == cudaSuccess) e = cudaMalloc(&s->tables, sizeof(double) * ntab);
      if (e == cudaSuccess)
        e = D == 2 ? fvh::plain::build_tables<2>(*mesh, s->tables, nnz[0], nnz[1], nnz[2], &s->tab)
                   : fvh::plain::build_tables<3>(*mesh, s->tables, nnz[0], nnz[1], nnz[2], &s->tab);
    } else {
      const fvh_status ms = fvh::mixed::create(*mesh, *params, &s->mixed);
      if (ms != FVH_OK) {
        fvh_solver_destroy(s);
        return ms;
      }
    }
    if (e == cudaSuccess)
      e = cudaMalloc(&s->scalars, sizeof(double) * 2 + fvh_time_step_workspace_bytes(mesh->num_cells));
    if (e == cudaSuccess) e = cudaMalloc(&s->status, sizeof(fvh_device_status));
    if (e == cudaSuccess) e = cudaMallocHost(&s->host_scalars, sizeof(double) * 2);
    if (e == cudaSuccess) e = cudaMallocHost(&s->host_status, sizeof(fvh_device_status));
    if (e == cudaSuccess) e = cudaMemset(s->scalars, 0, sizeof(double) * 2);
    if (e == cudaSuccess) e = cudaMemset(s->status, 0xff, sizeof(fvh_device_status));
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      fvh_solver_destroy(s);
      return from_cuda(e);
    }
    *out = s;
    return FVH_OK;
  });
}

static fvh_status solver_step_enqueue(fvh_solver *s, const fvh_state_view *state,
                                      cudaStream_t st,
                                      const fvh::mixed::launch_mark &mark = {},
                                      fvh::mixed::step_flags f = {}) {
  const fvh_mesh_view &m = s->mesh;
  const fvh_params &p = s->params;
  double *t = s->scalars, *dt = s->scalars + 1, *partial = s->scalars + 2;
  if (p.precision == FVH_PRECISION_MIXED)
    return from_cuda(fvh::mixed::step(s->mixed, m, p, *state, t, dt, partial,
                                      dt_blocks(m.num_cells), s->status, st, mark, s->shape, f));
  const fvh_stream_t fs = reinterpret_cast<fvh_stream_t>(st);
  const int nb = dt_blocks(m.num_cells);
  fvh_status r = from_cuda(
      m.dim == 2 ? fvh::plain::launch_dt<2>(m, *state, p, t, dt, partial, nb, s->status, st,
                                            s->tab.slot_dx, f.src)
                 : fvh::plain::launch_dt<3>(m, *state, p, t, dt, partial, nb, s->status, st,
                                            s->tab.slot_dx, f.src));
  mark("dt");
  for (int stage = 0; stage < 2 && r == FVH_OK; ++stage) {
    if (p.order == 1)
      r = fvh_evaluate_gradients(&m, state, &s->grads, &p, fs);
    else
      r = from_cuda(m.dim == 2
                        ? fvh::plain::launch_gradients<2>(m, *state, s->grads, p, st, s->tab)
                        : fvh::plain::launch_gradients<3>(m, *state, s->grads, p, st, s->tab));
    mark("gradients");
    if (r == FVH_OK)
      r = from_cuda(m.dim == 2
                        ? fvh::plain::launch_fluxes<2>(m, *state, s->grads, s->flux, p, st, s->tab)
                        : fvh::plain::launch_fluxes<3>(m, *state, s->grads, s->flux, p, st, s->tab));
    mark("fluxes");
    // the last stage of the step may also write the new state to f.out
    const fvh_state_view *out = stage == 1 ? f.out : nullptr;
    if (r == FVH_OK)
      r = from_cuda(m.dim == 2 ? fvh::plain::launch_update<2>(m, p, dt, 0.5, s->flux, *state, t,
                                                              s->status, st, out)
                               : fvh::plain::launch_update<3>(m, p, dt, 0.5, s->flux, *state, t,
                                                              s->status, st, out));
    mark("update");
  }
  return r;
}

// Flags of step k of a chunk of n consecutive steps: the first recomputes the
// pack and dt from the FP64 state, every corrector but the last writes them
// for the following step.
static fvh::mixed::step_flags chunk_flags(int64_t k, int64_t n) {
  fvh::mixed::step_flags f;
  f.pack_first = k == 0;
  f.write_next = k + 1 < n;
  return f;
}

static fvh_status solver_step_flags(fvh_solver *s, const fvh_state_view *state, cudaStream_t st,
                                    fvh::mixed::step_flags f);

fvh_status fvh_solver_set_shape(fvh_solver *s, int32_t block, int32_t cells_per_thread,
                                int32_t schedule) {
  const bool staged = (schedule & FVH_SCHEDULE_STAGED) != 0;
  schedule &= ~FVH_SCHEDULE_STAGED;
  if (!s || (block != 128 && block != 256) || cells_per_thread < 1 || cells_per_thread > 8 ||
      schedule < 0 || schedule > 2 ||
      (schedule == 2 && fvh::mixed::colours(s->mixed) == 0) ||
      (staged && !fvh::mixed::staging(s->mixed)))
    return FVH_ERR_INVALID_ARGUMENT;
  s->shape.block = block;
  s->shape.cells_per_thread = cells_per_thread;
  s->shape.schedule = schedule;
  s->shape.staged = staged;
  drop_graphs(s);
  return FVH_OK;
}

fvh_status fvh_solver_autotune(fvh_solver *s, const fvh_state_view *state, int32_t trial_steps,
                               int32_t *block, int32_t *cells_per_thread, int32_t *schedule,
                               double *best_ms_per_step, fvh_stream_t stream) {
  if (!s || !state_ok(state, s->mesh.dim) || trial_steps <= 0) return FVH_ERR_INVALID_ARGUMENT;
  if (s->params.precision != FVH_PRECISION_MIXED) {  // the FP64 path has one shape
    if (block) *block = 128;
    if (cells_per_thread) *cells_per_thread = 1;
    if (schedule) *schedule = 0;
    if (best_ms_per_step) *best_ms_per_step = -1;
    return FVH_OK;
  }
  cudaStream_t st = cs(stream);
  const int D = s->mesh.dim;
  const size_t nc = s->mesh.num_cells;
  // trials run on a scratch copy of the state; the caller's state, solution
  // time and status word are left as they were
  double *scratch = nullptr, *saved_t = nullptr;
  cudaError_t e = cudaMalloc(&scratch, sizeof(double) * (5 + D) * nc);
  if (e == cudaSuccess) e = cudaMalloc(&saved_t, sizeof(double) + sizeof(fvh_device_status));
  if (e != cudaSuccess) {
    cudaFree(scratch);
    return from_cuda(e);
  }
  double *planes_src[9], *planes_dst[9];
  fvh_state_view tmp{};
  {
    int k = 0;
    planes_src[k++] = state->density;
    for (int d = 0; d < D; ++d) planes_src[k++] = state->velocity[d];
    planes_src[k++] = state->internal_energy;
    planes_src[k++] = state->pressure;
    planes_src[k++] = state->temperature;
    planes_src[k++] = state->sound_speed;
    for (int q = 0; q < 5 + D; ++q) planes_dst[q] = scratch + q * nc;
    k = 0;
    tmp.density = planes_dst[k++];
    for (int d = 0; d < D; ++d) tmp.velocity[d] = planes_dst[k++];
    tmp.internal_energy = planes_dst[k++];
    tmp.pressure = planes_dst[k++];
    tmp.temperature = planes_dst[k++];
    tmp.sound_speed = planes_dst[k++];
  }
  e = cudaMemcpyAsync(saved_t, s->scalars, sizeof(double), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(saved_t + 1, s->status, sizeof(fvh_device_status), cudaMemcpyDeviceToDevice, st);
  auto refresh = [&]() {
    for (int q = 0; q < 5 + D && e == cudaSuccess; ++q)
      e = cudaMemcpyAsync(planes_dst[q], planes_src[q], sizeof(double) * nc,
                          cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->scalars, saved_t, sizeof(double), cudaMemcpyDeviceToDevice, st);
  };
  const fvh::mixed::launch_shape keep = s->shape;
  fvh::mixed::launch_shape best = keep;
  double best_ms = -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // every shape timed in each of kAutotuneRounds interleaved rounds; a shape's
  // figure is its fastest round (robust to a one-off slow trial)
  // each shape with the global-memory gradients, and where the mesh allows
  // it with the staged ones
  constexpr int NB = fvh::mixed::kNumShapes;
  const int NS = fvh::mixed::staging(s->mixed) ? 2 * NB : NB;
  auto shape_at = [&](int i) {
    fvh::mixed::launch_shape c = fvh::mixed::kShapes[i % NB];
    c.staged = i >= NB;
    return c;
  };
  double shape_ms[2 * NB];
  for (int i = 0; i < NS; ++i) shape_ms[i] = -1;
  for (int round = 0; round < fvh::mixed::kAutotuneRounds; ++round) {
    for (int i = 0; i < NS; ++i) {
      const auto c = shape_at(i);
      if (e != cudaSuccess) break;
      fvh_solver_set_shape(s, c.block, c.cells_per_thread,
                           c.schedule | (c.staged ? FVH_SCHEDULE_STAGED : 0));
      refresh();
      // timed as fvh_solver_run launches steps
      fvh_status r = FVH_OK;
      for (int k = 0; k < trial_steps && r == FVH_OK; ++k)
        r = solver_step_flags(s, &tmp, st, chunk_flags(k, trial_steps));
      refresh();
      cudaEventRecord(e0, st);
      for (int k = 0; k < trial_steps && r == FVH_OK; ++k)
        r = solver_step_flags(s, &tmp, st, chunk_flags(k, trial_steps));
      cudaEventRecord(e1, st);
      if (r == FVH_OK) e = cudaEventSynchronize(e1);
      if (r != FVH_OK || e != cudaSuccess) continue;
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      const double per = ms / trial_steps;
      if (shape_ms[i] < 0 || per < shape_ms[i]) shape_ms[i] = per;
    }
  }
  for (int i = 0; i < NS; ++i)
    if (shape_ms[i] >= 0 && (best_ms < 0 || shape_ms[i] < best_ms)) {
      best_ms = shape_ms[i];
      best = shape_at(i);
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->scalars, saved_t, sizeof(double), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->status, saved_t + 1, sizeof(fvh_device_status), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(scratch);
  cudaFree(saved_t);
  fvh_solver_set_shape(s, best.block, best.cells_per_thread,
                       best.schedule | (best.staged ? FVH_SCHEDULE_STAGED : 0));
  if (e != cudaSuccess) return from_cuda(e);
  if (block) *block = best.block;
  if (cells_per_thread) *cells_per_thread = best.cells_per_thread;
  if (schedule) *schedule = best.schedule | (best.staged ? FVH_SCHEDULE_STAGED : 0);
  if (best_ms_per_step) *best_ms_per_step = best_ms;
  return FVH_OK;
}

fvh_status fvh_debug_split(const double *x, int64_t n, float *hi, float *lo, float *rn32,
                           double *hi_as_double, fvh_stream_t stream) {
  if (n < 0 || (n > 0 && (!x || !hi || !lo || !rn32 || !hi_as_double)))
    return FVH_ERR_INVALID_ARGUMENT;
  return from_cuda(fvh::mixed::debug_split(x, n, hi, lo, rn32, hi_as_double, cs(stream)));
}

fvh_status fvh_debug_sf64(int32_t op, const double *a, const double *b, int64_t n,
                          double *out, fvh_stream_t stream) {
  if (op < 0 || op > 10 || n < 0 || (n > 0 && (!a || !b || !out)))
    return FVH_ERR_INVALID_ARGUMENT;
  return from_cuda(fvh::plain::debug_sf64(op, a, b, n, out, cs(stream)));
}

int64_t fvh_solver_launches_per_run(const fvh_solver *s, int64_t nsteps) {
  if (!s || nsteps <= 0) return 0;
  if (s->params.precision != FVH_PRECISION_MIXED)
    return nsteps * fvh_solver_launches_per_step(s);
  int64_t total = 0;
  for (int64_t k = 0; k < nsteps && k < 2; ++k)  // the first step and one of the rest
    total += fvh::mixed::launches_per_step(s->params, s->shape, chunk_flags(k, nsteps),
                                           fvh::mixed::colours(s->mixed));
  if (nsteps > 2)
    total += (nsteps - 2) * fvh::mixed::launches_per_step(s->params, s->shape,
                                                          chunk_flags(1, nsteps),
                                                          fvh::mixed::colours(s->mixed));
  return total;
}

int32_t fvh_solver_launches_per_step(const fvh_solver *s) {
  if (!s) return 0;
  if (s->params.precision == FVH_PRECISION_MIXED)
    return fvh::mixed::launches_per_step(s->params, s->shape, {},
                                         fvh::mixed::colours(s->mixed));
  // dt (partial + final) + per stage: gradients (or D*(D+4) memsets), fluxes, update
  const int D = s->mesh.dim;
  const int grad = s->params.order == 1 ? D * (D + 4) : 1;
  return 2 + 2 * (grad + 2);
}

namespace {
struct profile_ctx {
  cudaStream_t st;
  std::vector<cudaEvent_t> events;
  std::vector<const char *> names;
  size_t next = 0;
};
void profile_mark(void *vctx, const char *name) {
  profile_ctx *c = static_cast<profile_ctx *>(vctx);
  if (c->next < c->events.size()) {
    cudaEventRecord(c->events[c->next], c->st);
    c->names.push_back(name);
  }
  c->next++;
}
}  // namespace

fvh_status fvh_solver_profile(fvh_solver *s, const fvh_state_view *state, int32_t nsteps,
                              int32_t max_kernels, const char **names, double *mean_ms,
                              int32_t *launches, int32_t *nkernels, fvh_stream_t stream) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!s || !state_ok(state, s->mesh.dim) || nsteps <= 0 || max_kernels <= 0 || !names ||
        !mean_ms || !launches || !nkernels)
      return FVH_ERR_INVALID_ARGUMENT;
    profile_ctx ctx;
    ctx.st = cs(stream);
    const size_t nev = (size_t)nsteps * 16 + 1;
    ctx.events.resize(nev);
    ctx.names.reserve(nev);  // profile_mark records at most nev names, without reallocating
    std::vector<double> total(max_kernels, 0.0);
    std::vector<int> count(max_kernels, 0);
    for (auto &e : ctx.events) cudaEventCreate(&e);  // nothing below allocates host memory
    fvh::mixed::launch_mark mark;
    mark.fn = profile_mark;
    mark.ctx = &ctx;
    fvh_status r = FVH_OK;
    profile_mark(&ctx, "");  // start event
    for (int k = 0; k < nsteps && r == FVH_OK; ++k)
      r = solver_step_enqueue(s, state, ctx.st, mark, chunk_flags(k, nsteps));
    if (r == FVH_OK) r = from_cuda(cudaStreamSynchronize(ctx.st));
    int32_t nk = 0;
    if (r == FVH_OK) {
      const size_t recorded = ctx.names.size();
      for (size_t i = 1; i < recorded; ++i) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx.events[i - 1], ctx.events[i]);
        int k = 0;
        for (; k < nk; ++k)
          if (std::strcmp(names[k], ctx.names[i]) == 0) break;
        if (k == nk) {
          if (nk == max_kernels) continue;
          names[nk++] = ctx.names[i];
        }
        total[k] += ms;
        count[k]++;
      }
      for (int k = 0; k < nk; ++k) {
        mean_ms[k] = count[k] ? total[k] / count[k] : 0.0;
        launches[k] = count[k];
      }
    }
    *nkernels = nk;
    for (auto &e : ctx.events) cudaEventDestroy(e);
    return r;
  });
}

// One step is a fixed sequence of launches; each variant is captured once per
// (stream, state) into a CUDA graph and replayed.
static fvh_status solver_step_flags(fvh_solver *s, const fvh_state_view *state, cudaStream_t st,
                                    fvh::mixed::step_flags f) {
  if (s->params.precision != FVH_PRECISION_MIXED) f = fvh::mixed::step_flags();
  if (st == nullptr) return solver_step_enqueue(s, state, st, {}, f);
  if (s->graph_stream != st || std::memcmp(&s->graph_state, state, sizeof(*state)) != 0) {
    drop_graphs(s);
    s->graph_stream = st;
    s->graph_state = *state;
  }
  cudaGraphExec_t &ge = s->graph[(f.pack_first ? 2 : 0) + (f.write_next ? 1 : 0)];
  if (!ge) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return from_cuda(e);
    const fvh_status r = solver_step_enqueue(s, state, st, {}, f);
    e = cudaStreamEndCapture(st, &g);
    if (r != FVH_OK) {
      if (g) cudaGraphDestroy(g);
      return r;
    }
    if (e != cudaSuccess) return from_cuda(e);
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      ge = nullptr;
      return from_cuda(e);
    }
  }
  return from_cuda(cudaGraphLaunch(ge, st));
}

fvh_status fvh_solver_step(fvh_solver *s, const fvh_state_view *state, fvh_stream_t stream) {
  if (!s || !state_ok(state, s->mesh.dim)) return FVH_ERR_INVALID_ARGUMENT;
  return solver_step_flags(s, state, cs(stream), fvh::mixed::step_flags());
}

fvh_status fvh_solver_check(fvh_solver *s, fvh_stream_t stream, double *soln_time,
                            int64_t *bad_cell) {
  if (!s) return FVH_ERR_INVALID_ARGUMENT;
  cudaStream_t st = cs(stream);
  cudaMemcpyAsync(s->host_scalars, s->scalars, sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(s->host_status, s->status, sizeof(fvh_device_status), cudaMemcpyDeviceToHost,
                  st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return from_cuda(e);
  if (soln_time) *soln_time = s->host_scalars[0];
  int32_t code;
  int64_t cell;
  fvh_status_decode(*s->host_status, &code, &cell);
  if (bad_cell) *bad_cell = cell;
  return (fvh_status)code;
}

fvh_status fvh_solver_reset(fvh_solver *s, double t, fvh_stream_t stream) {
  if (!s) return FVH_ERR_INVALID_ARGUMENT;
  cudaStream_t st = cs(stream);
  s->host_scalars[1] = t;
  cudaError_t e = cudaMemcpyAsync(s->scalars, s->host_scalars + 1, sizeof(double),
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->status, 0xff, sizeof(fvh_device_status), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return from_cuda(e);
}

fvh_status fvh_solver_run(fvh_solver *s, const fvh_state_view *state, int64_t nsteps,
                          int32_t stop_at_final_time, int32_t check_every,
                          int64_t *steps_done, fvh_stream_t stream) {
  if (!s || !state_ok(state, s->mesh.dim) || nsteps < 0) return FVH_ERR_INVALID_ARGUMENT;
  if (check_every <= 0) check_every = 1;
  int64_t n = 0;
  fvh_status r = FVH_OK;
  const double tf = s->params.final_time;
  const double t_stop = tf - 1e-12 * std::fabs(tf);
  while (n < nsteps) {
    if (stop_at_final_time) {
      double t = 0;
      r = fvh_solver_check(s, stream, &t, nullptr);
      if (r != FVH_OK || t >= t_stop) break;
    }
    const int64_t chunk = stop_at_final_time
                              ? (nsteps - n < check_every ? nsteps - n : check_every)
                              : nsteps - n;
    for (int64_t k = 0; k < chunk && r == FVH_OK; ++k, ++n)
      r = solver_step_flags(s, state, cs(stream), chunk_flags(k, chunk));
    if (r != FVH_OK) break;
  }
  if (r == FVH_OK) r = fvh_solver_check(s, stream, nullptr, nullptr);
  if (steps_done) *steps_done = n;
  return r;
}

double *fvh_solver_soln_time(fvh_solver *s) { return s ? s->scalars : nullptr; }
double *fvh_solver_dt(fvh_solver *s) { return s ? s->scalars + 1 : nullptr; }
fvh_device_status *fvh_solver_status(fvh_solver *s) { return s ? s->status : nullptr; }
const fvh_gradient_view *fvh_solver_gradients(fvh_solver *s) {
  if (!s) return nullptr;
  return s->params.precision == FVH_PRECISION_FP64 ? &s->grads : nullptr;
}
const fvh_flux_view *fvh_solver_fluxes(fvh_solver *s) {
  if (!s) return nullptr;
  return s->params.precision == FVH_PRECISION_FP64 ? &s->flux : nullptr;
}

// ---------------------------------------------------------------------------
// device memory helpers
// ---------------------------------------------------------------------------
void fvh_device_mesh_destroy(fvh_device_mesh *dm) {
  if (!dm) return;
  for (void *p : dm->allocs) cudaFree(p);
  delete dm;
}

fvh_status fvh_device_mesh_create(const fvh_host_mesh *m, fvh_device_mesh **out) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!m || !out) return FVH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    fvh_device_mesh *dm = new (std::nothrow) fvh_device_mesh();
    if (!dm) return FVH_ERR_OUT_OF_MEMORY;
    std::unique_ptr<fvh_device_mesh, void (*)(fvh_device_mesh *)> own(dm, fvh_device_mesh_destroy);
    dm->allocs.reserve(32);  // at most 21 arrays: recording one never throws
    cudaError_t e = cudaSuccess;
    auto up = [&](const void *src, size_t bytes) -> void * {
      if (e != cudaSuccess) return nullptr;
      void *d = nullptr;
      e = cudaMalloc(&d, bytes > 0 ? bytes : 16);
      if (e != cudaSuccess) return nullptr;
      dm->allocs.push_back(d);
      if (bytes) e = cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice);
      return d;
    };
    auto upi = [&](const std::vector<int32_t> &v) {
      return static_cast<const int32_t *>(up(v.data(), v.size() * sizeof(int32_t)));
    };
    auto upd = [&](const std::vector<double> &v) {
      return static_cast<const double *>(up(v.data(), v.size() * sizeof(double)));
    };
    fvh_mesh_view &o = dm->view;
    dm->nnz_cf = (int32_t)m->cf.size();
    dm->nnz_nb = (int32_t)m->nb.size();
    dm->nnz_cv = (int32_t)m->cv.size();
    o.dim = m->dim;
    o.num_cells = m->nc;
    o.num_faces = m->nf;
    o.num_vertices = m->nv;
    o.face_cells = upi(m->face_cells);
    o.cell_face_offsets = upi(m->cf_off);
    o.cell_faces = upi(m->cf);
    o.cell_nbr_offsets = upi(m->nb_off);
    o.cell_nbrs = upi(m->nb);
    o.cell_vertex_offsets = upi(m->cv_off);
    o.cell_vertices = upi(m->cv);
    for (int d = 0; d < m->dim; ++d) {
      o.cell_centroid[d] = upd(m->cc[d]);
      o.face_centroid[d] = upd(m->fc[d]);
      o.face_normal[d] = upd(m->fn[d]);
      o.vertex_coord[d] = upd(m->vc[d]);
    }
    o.cell_volume = upd(m->cvol);
    o.face_area = upd(m->fa);
    if (e != cudaSuccess) return from_cuda(e);
    *out = own.release();
    return FVH_OK;
  });
}

const fvh_mesh_view *fvh_device_mesh_view(const fvh_device_mesh *dm) {
  return dm ? &dm->view : nullptr;
}

void fvh_device_state_destroy(fvh_device_state *ds) {
  if (!ds) return;
  cudaFree(ds->base);
  delete ds;
}

fvh_status fvh_device_state_create(int32_t dim, int32_t num_cells, fvh_device_state **out) {
  if (!out || (dim != 2 && dim != 3) || num_cells <= 0) return FVH_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  fvh_device_state *ds = new (std::nothrow) fvh_device_state();
  if (!ds) return FVH_ERR_OUT_OF_MEMORY;
  // planes padded to 64 doubles so each starts on a 512-byte boundary
  const size_t stride = ((size_t)num_cells + 63) / 64 * 64;
  const cudaError_t e = cudaMalloc(&ds->base, sizeof(double) * stride * (5 + dim));
  if (e != cudaSuccess) {
    delete ds;
    return from_cuda(e);
  }
  double *b = ds->base;
  ds->view.density = b;
  b += stride;
  for (int d = 0; d < dim; ++d, b += stride) ds->view.velocity[d] = b;
  ds->view.internal_energy = b;
  b += stride;
  ds->view.pressure = b;
  b += stride;
  ds->view.temperature = b;
  b += stride;
  ds->view.sound_speed = b;
  *out = ds;
  return FVH_OK;
}

const fvh_state_view *fvh_device_state_view(const fvh_device_state *ds) {
  return ds ? &ds->view : nullptr;
}

static void state_planes(const fvh_state_view *s, int dim, double **p) {
  int k = 0;
  p[k++] = s->density;
  for (int d = 0; d < dim; ++d) p[k++] = s->velocity[d];
  p[k++] = s->internal_energy;
  p[k++] = s->pressure;
  p[k++] = s->temperature;
  p[k++] = s->sound_speed;
}

fvh_status fvh_state_upload(const fvh_state_view *dst, int32_t dim, int32_t num_cells,
                            const double *host, fvh_stream_t stream) {
  if (!state_ok(dst, dim) || !host || num_cells <= 0) return FVH_ERR_INVALID_ARGUMENT;
  double *planes[9];
  state_planes(dst, dim, planes);
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 5 + dim && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(planes[k], host + (size_t)k * num_cells, sizeof(double) * num_cells,
                        cudaMemcpyHostToDevice, cs(stream));
  return from_cuda(e);
}

fvh_status fvh_state_download(const fvh_state_view *src, int32_t dim, int32_t num_cells,
                              double *host, fvh_stream_t stream) {
  if (!state_ok(src, dim) || !host || num_cells <= 0) return FVH_ERR_INVALID_ARGUMENT;
  double *planes[9];
  state_planes(src, dim, planes);
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 5 + dim && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(host + (size_t)k * num_cells, planes[k], sizeof(double) * num_cells,
                        cudaMemcpyDeviceToHost, cs(stream));
  return from_cuda(e);
}

fvh_status fvh_solver_advance_host(fvh_solver *s, const fvh_state_view *dev_state,
                                   double *host_planes, int64_t nsteps, double *soln_time,
                                   fvh_stream_t stream) {
  if (!s || !state_ok(dev_state, s->mesh.dim) || !host_planes || !soln_time || nsteps < 0)
    return FVH_ERR_INVALID_ARGUMENT;
  const int D = s->mesh.dim, nc = s->mesh.num_cells;
  cudaStream_t st = cs(stream);
  s->host_scalars[1] = *soln_time;
  cudaError_t e = cudaMemcpyAsync(s->scalars, s->host_scalars + 1, sizeof(double),
                                  cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return from_cuda(e);
  // Pinned (device-mapped) host planes: the first kernel (the mixed form's
  // pack_dt, the FP64 form's dt) reads the state straight from host memory,
  // storing it into the device state as it goes, and the last update writes
  // the new state back to host memory while it computes, so the transfers
  // overlap the kernels instead of preceding and following them.
  cudaPointerAttributes attr{};
  if (nsteps > 0 && cudaPointerGetAttributes(&attr, host_planes) == cudaSuccess &&
      attr.type == cudaMemoryTypeHost && attr.devicePointer) {
    double *hp = static_cast<double *>(attr.devicePointer);
    fvh_state_view hv{};
    int k = 0;
    hv.density = hp + (size_t)k++ * nc;
    for (int d = 0; d < D; ++d) hv.velocity[d] = hp + (size_t)k++ * nc;
    hv.internal_energy = hp + (size_t)k++ * nc;
    hv.pressure = hp + (size_t)k++ * nc;
    hv.temperature = hp + (size_t)k++ * nc;
    hv.sound_speed = hp + (size_t)k++ * nc;
    fvh_status r = FVH_OK;
    for (int64_t n = 0; n < nsteps && r == FVH_OK; ++n) {
      fvh::mixed::step_flags f = chunk_flags(n, nsteps);
      if (n == 0) f.src = &hv;
      if (n + 1 == nsteps) f.out = &hv;
      r = solver_step_enqueue(s, dev_state, st, {}, f);
    }
    if (r != FVH_OK) return r;
    double t = 0;
    r = fvh_solver_check(s, stream, &t, nullptr);
    *soln_time = t;
    return r;
  }
  cudaGetLastError();  // a pageable pointer is not an error
  fvh_status r = fvh_state_upload(dev_state, D, nc, host_planes, stream);
  for (int64_t k = 0; k < nsteps && r == FVH_OK; ++k) r = fvh_solver_step(s, dev_state, stream);
  if (r == FVH_OK) r = fvh_state_download(dev_state, D, nc, host_planes, stream);
  if (r != FVH_OK) return r;
  double t = 0;
  r = fvh_solver_check(s, stream, &t, nullptr);
  *soln_time = t;
  return r;
}

}  // extern "C"
