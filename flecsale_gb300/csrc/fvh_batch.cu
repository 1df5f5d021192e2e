// Batched form: many independent meshes advanced together.
//
// The problems of an assignment are concatenated into one block-diagonal mesh
// (fvh_host_mesh_concat) held in buffers sized once for a capacity, so the set
// of problems can change between launches without reallocating (continuous
// batching).  One step of every problem is the mixed-precision step with a
// per-problem CFL dt (segmented maximum), per-problem solution time and status;
// problems that reached their final time get dt = 0 and stay unchanged.  Steps
// are captured into one CUDA graph per (stream, step count) and replayed.
// Because a problem's cells only read cells of the same problem and its dt is
// a maximum over its own cells, every problem's result is the same whatever
// else is in the batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "flecsale_gb300.h"
#include "fvh_internal.h"
#include "fvh_kernels.h"
#include "fvh_mixed.h"

namespace {

inline fvh_status from_cuda(cudaError_t e) {
  if (e == cudaSuccess) return FVH_OK;
  if (e == cudaErrorMemoryAllocation) return FVH_ERR_OUT_OF_MEMORY;
  return FVH_ERR_CUDA;
}

// The launch shapes the batch kernels support: fvh_batch_set_shape accepts
// only these, and a cached entry outside them (a damaged or hand-edited cache
// file) is ignored rather than launched.
bool batch_shape_ok(int block, int cells_per_thread, int schedule) {
  return (block == 128 || block == 256) && cells_per_thread >= 1 && cells_per_thread <= 8 &&
         (schedule == 0 || schedule == 1);
}

}  // namespace

struct fvh_batch {
  fvh_params params{};
  int dim = 0;
  // capacities
  int64_t max_cells = 0, max_faces = 0, max_vertices = 0;
  int64_t max_cf = 0, max_nb = 0, max_cv = 0;
  int32_t max_problems = 0;
  // device mesh arrays (capacity-sized)
  std::vector<void *> allocs;
  int32_t *face_cells = nullptr, *cf_off = nullptr, *cf = nullptr, *nb_off = nullptr,
          *nb = nullptr, *cv_off = nullptr, *cv = nullptr;
  double *geo = nullptr;  // cell centroid[D], volume, face centroid[D], normal[D], area, vertex[D]
  fvh_mesh_view view{};
  // state: two buffers so a re-assignment can move states without overlap
  double *state_buf[2] = {nullptr, nullptr};
  int cur = 0;
  fvh_state_view state{};
  // problems
  int32_t nproblems = 0;
  std::vector<int32_t> first_cell;  // host copy [P+1]
  int32_t *cell_problem = nullptr, *d_first_cell = nullptr;
  double *cfl = nullptr, *tf = nullptr, *t = nullptr, *dt = nullptr;
  unsigned *dtinv_bits = nullptr;
  fvh_device_status *status = nullptr;
  fvh::mixed::workspace *ws = nullptr;
  fvh::mixed::launch_shape shape;
  // pinned staging for queries
  double *h_t = nullptr;
  fvh_device_status *h_status = nullptr;
  // graphs keyed by step count (for one stream)
  cudaStream_t graph_stream = nullptr;
  std::map<int, cudaGraphExec_t> graphs;
};

namespace {

void drop_graphs(fvh_batch *b) {
  for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
}

fvh::mixed::problem_map pmap(const fvh_batch *b) {
  fvh::mixed::problem_map pm;
  pm.cell_problem = b->cell_problem;
  pm.first_cell = b->d_first_cell;
  pm.nproblems = b->nproblems;
  pm.cfl = b->cfl;
  pm.final_time = b->tf;
  pm.t = b->t;
  pm.dt = b->dt;
  pm.dtinv_bits = b->dtinv_bits;
  pm.status = b->status;
  return pm;
}

void set_state_view(fvh_batch *b) {
  const int64_t stride = b->max_cells;
  double *base = b->state_buf[b->cur];
  fvh_state_view &s = b->state;
  std::memset(&s, 0, sizeof(s));
  int k = 0;
  s.density = base + stride * k++;
  for (int d = 0; d < b->dim; ++d) s.velocity[d] = base + stride * k++;
  s.internal_energy = base + stride * k++;
  s.pressure = base + stride * k++;
  s.temperature = base + stride * k++;
  s.sound_speed = base + stride * k++;
}

// A reassignment that failed after it began to overwrite the batch's device
// arrays leaves no consistent problem set: the batch is emptied (no problems,
// no graphs), so fvh_batch_step refuses to run until the next successful
// assignment instead of stepping a mix of old and new meshes.
fvh_status fail_assign(fvh_batch *b, cudaError_t e) {
  drop_graphs(b);
  b->nproblems = 0;
  b->first_cell.assign(1, 0);
  std::memset(&b->view, 0, sizeof(b->view));
  b->view.dim = b->dim;
  return from_cuda(e);
}

}  // namespace

extern "C" {

void fvh_batch_destroy(fvh_batch *b) {
  if (!b) return;
  drop_graphs(b);
  if (b->ws) fvh::mixed::destroy(b->ws);
  for (void *p : b->allocs) cudaFree(p);
  cudaFreeHost(b->h_t);
  cudaFreeHost(b->h_status);
  delete b;
}

fvh_status fvh_batch_create(const fvh_params *params, int64_t max_cells, int64_t max_faces,
                            int64_t max_vertices, int32_t max_problems, fvh_batch **out) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!out || !params || (params->dim != 2 && params->dim != 3) || max_cells <= 0 ||
        max_faces <= 0 || max_vertices <= 0 || max_problems <= 0 ||
        params->precision != FVH_PRECISION_MIXED || !(params->gamma > 1) || !(params->cv > 0))
      return FVH_ERR_INVALID_ARGUMENT;
    if (max_cells >= INT32_MAX / 26 || max_faces >= INT32_MAX / 2 || max_vertices >= INT32_MAX)
      return FVH_ERR_CAPACITY;
    *out = nullptr;
    fvh_batch *b = new (std::nothrow) fvh_batch();
    if (!b) return FVH_ERR_OUT_OF_MEMORY;
    std::unique_ptr<fvh_batch, void (*)(fvh_batch *)> own(b, fvh_batch_destroy);
    b->allocs.reserve(32);  // 18 device arrays: recording one never throws
    b->params = *params;
    const int D = b->dim = params->dim;
    b->max_cells = max_cells;
    b->max_faces = max_faces;
    b->max_vertices = max_vertices;
    b->max_problems = max_problems;
    b->max_cf = max_cells * (D == 2 ? 6 : 6);
    b->max_nb = max_cells * (D == 2 ? 12 : 26);
    b->max_cv = max_cells * (D == 2 ? 6 : 8);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](size_t bytes) -> void * {
      void *p = nullptr;
      if (e == cudaSuccess) e = cudaMalloc(&p, bytes > 0 ? bytes : 16);
      if (e == cudaSuccess) b->allocs.push_back(p);
      return p;
    };
    b->face_cells = static_cast<int32_t *>(alloc(sizeof(int32_t) * 2 * max_faces));
    b->cf_off = static_cast<int32_t *>(alloc(sizeof(int32_t) * (max_cells + 1)));
    b->cf = static_cast<int32_t *>(alloc(sizeof(int32_t) * b->max_cf));
    b->nb_off = static_cast<int32_t *>(alloc(sizeof(int32_t) * (max_cells + 1)));
    b->nb = static_cast<int32_t *>(alloc(sizeof(int32_t) * b->max_nb));
    b->cv_off = static_cast<int32_t *>(alloc(sizeof(int32_t) * (max_cells + 1)));
    b->cv = static_cast<int32_t *>(alloc(sizeof(int32_t) * b->max_cv));
    b->geo = static_cast<double *>(alloc(sizeof(double) * ((size_t)(D + 1) * max_cells +
                                                          (size_t)(2 * D + 1) * max_faces +
                                                          (size_t)D * max_vertices)));
    for (int k = 0; k < 2; ++k)
      b->state_buf[k] = static_cast<double *>(alloc(sizeof(double) * (5 + D) * max_cells));
    b->cell_problem = static_cast<int32_t *>(alloc(sizeof(int32_t) * max_cells));
    b->d_first_cell = static_cast<int32_t *>(alloc(sizeof(int32_t) * (max_problems + 1)));
    b->cfl = static_cast<double *>(alloc(sizeof(double) * max_problems));
    b->tf = static_cast<double *>(alloc(sizeof(double) * max_problems));
    b->t = static_cast<double *>(alloc(sizeof(double) * max_problems));
    b->dt = static_cast<double *>(alloc(sizeof(double) * max_problems));
    b->dtinv_bits = static_cast<unsigned *>(alloc(sizeof(unsigned) * max_problems));
    b->status = static_cast<fvh_device_status *>(alloc(sizeof(fvh_device_status) * max_problems));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_t, sizeof(double) * max_problems);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_status, sizeof(fvh_device_status) * max_problems);
    if (e == cudaSuccess) e = cudaMemset(b->dtinv_bits, 0, sizeof(unsigned) * max_problems);
    if (e == cudaSuccess) e = cudaMemset(b->status, 0xff, sizeof(fvh_device_status) * max_problems);
    if (e != cudaSuccess) return from_cuda(e);
    const fvh_status r = fvh::mixed::create_capacity(D, max_cells, max_faces, max_vertices, &b->ws);
    if (r != FVH_OK) return r;
    set_state_view(b);
    *out = own.release();
    return FVH_OK;
  });
}

fvh_status fvh_batch_assign(fvh_batch *b, int32_t n, const fvh_host_mesh *const *meshes,
                            const double *cfl, const double *final_time, const int32_t *keep,
                            fvh_stream_t stream) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!b || n <= 0 || !meshes || !cfl || !final_time) return FVH_ERR_INVALID_ARGUMENT;
    if (n > b->max_problems) return FVH_ERR_CAPACITY;
    for (int k = 0; k < n; ++k)
      if (!meshes[k] || meshes[k]->dim != b->dim || !(cfl[k] > 0)) return FVH_ERR_INVALID_ARGUMENT;
    // a carried problem must exist and keep its cell count; checked before any
    // device memory is touched
    if (keep)
      for (int k = 0; k < n; ++k) {
        if (keep[k] >= b->nproblems) return FVH_ERR_INVALID_ARGUMENT;
        if (keep[k] >= 0 &&
            b->first_cell[keep[k] + 1] - b->first_cell[keep[k]] != meshes[k]->nc)
          return FVH_ERR_INVALID_ARGUMENT;
      }
    fvh_host_mesh *cat = nullptr;
    fvh_status r = fvh_host_mesh_concat(n, meshes, &cat);
    if (r != FVH_OK) return r;
    std::unique_ptr<fvh_host_mesh, void (*)(fvh_host_mesh *)> own_cat(cat, fvh_host_mesh_destroy);
    const int D = b->dim;
    if (cat->nc > b->max_cells || cat->nf > b->max_faces || cat->nv > b->max_vertices ||
        (int64_t)cat->cf.size() > b->max_cf || (int64_t)cat->nb.size() > b->max_nb ||
        (int64_t)cat->cv.size() > b->max_cv)
      return FVH_ERR_CAPACITY;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    // states that carry over are gathered into the other buffer
    std::vector<int32_t> old_first = b->first_cell;
    std::vector<int32_t> first(n + 1, 0), cell_problem(cat->nc);
    for (int k = 0; k < n; ++k) {
      first[k + 1] = first[k] + meshes[k]->nc;
      for (int c = first[k]; c < first[k + 1]; ++c) cell_problem[c] = k;
    }
    cudaError_t e = cudaStreamSynchronize(st);  // previous steps done before overwriting
    const int nxt = 1 - b->cur;
    const int64_t stride = b->max_cells;
    std::vector<double> times(n, 0.0);
    if (e == cudaSuccess && keep && b->nproblems > 0)
      e = cudaMemcpy(b->h_t, b->t, sizeof(double) * b->nproblems, cudaMemcpyDeviceToHost);
    for (int k = 0; k < n && e == cudaSuccess; ++k) {
      if (!keep || keep[k] < 0) continue;
      const int o = keep[k];
      const int64_t ncells = old_first[o + 1] - old_first[o];  // == meshes[k]->nc
      times[k] = b->h_t[o];
      for (int pl = 0; pl < 5 + D && e == cudaSuccess; ++pl)
        e = cudaMemcpyAsync(b->state_buf[nxt] + pl * stride + first[k],
                            b->state_buf[b->cur] + pl * stride + old_first[o],
                            sizeof(double) * ncells, cudaMemcpyDeviceToDevice, st);
    }
    // mesh arrays
    auto up = [&](void *dst, const void *src, size_t bytes) {
      if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    up(b->face_cells, cat->face_cells.data(), sizeof(int32_t) * cat->face_cells.size());
    up(b->cf_off, cat->cf_off.data(), sizeof(int32_t) * cat->cf_off.size());
    up(b->cf, cat->cf.data(), sizeof(int32_t) * cat->cf.size());
    up(b->nb_off, cat->nb_off.data(), sizeof(int32_t) * cat->nb_off.size());
    up(b->nb, cat->nb.data(), sizeof(int32_t) * cat->nb.size());
    up(b->cv_off, cat->cv_off.data(), sizeof(int32_t) * cat->cv_off.size());
    up(b->cv, cat->cv.data(), sizeof(int32_t) * cat->cv.size());
    // the new view is committed to the batch only once everything succeeded
    fvh_mesh_view v;
    std::memset(&v, 0, sizeof(v));
    v.dim = D;
    v.num_cells = cat->nc;
    v.num_faces = cat->nf;
    v.num_vertices = cat->nv;
    v.face_cells = b->face_cells;
    v.cell_face_offsets = b->cf_off;
    v.cell_faces = b->cf;
    v.cell_nbr_offsets = b->nb_off;
    v.cell_nbrs = b->nb;
    v.cell_vertex_offsets = b->cv_off;
    v.cell_vertices = b->cv;
    double *g = b->geo;
    for (int d = 0; d < D; ++d, g += b->max_cells) {
      up(g, cat->cc[d].data(), sizeof(double) * cat->nc);
      v.cell_centroid[d] = g;
    }
    up(g, cat->cvol.data(), sizeof(double) * cat->nc);
    v.cell_volume = g;
    g += b->max_cells;
    for (int d = 0; d < D; ++d, g += b->max_faces) {
      up(g, cat->fc[d].data(), sizeof(double) * cat->nf);
      v.face_centroid[d] = g;
    }
    for (int d = 0; d < D; ++d, g += b->max_faces) {
      up(g, cat->fn[d].data(), sizeof(double) * cat->nf);
      v.face_normal[d] = g;
    }
    up(g, cat->fa.data(), sizeof(double) * cat->nf);
    v.face_area = g;
    g += b->max_faces;
    for (int d = 0; d < D; ++d, g += b->max_vertices) {
      up(g, cat->vc[d].data(), sizeof(double) * cat->nv);
      v.vertex_coord[d] = g;
    }
    // problems
    up(b->cell_problem, cell_problem.data(), sizeof(int32_t) * cat->nc);
    up(b->d_first_cell, first.data(), sizeof(int32_t) * (n + 1));
    up(b->cfl, cfl, sizeof(double) * n);
    up(b->tf, final_time, sizeof(double) * n);
    up(b->t, times.data(), sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dtinv_bits, 0, sizeof(unsigned) * n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->status, 0xff, sizeof(fvh_device_status) * n, st);
    if (e == cudaSuccess) e = fvh::mixed::setup_geometry(b->ws, v, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // before the host arrays are freed
    if (e != cudaSuccess) return fail_assign(b, e);
    b->view = v;
    b->cur = nxt;
    set_state_view(b);
    b->first_cell = std::move(first);
    b->nproblems = n;
    drop_graphs(b);
    return FVH_OK;
  });
}

// ---------------------------------------------------------------------------
// device-side assignment: problems already in device memory are concatenated
// by gather kernels (indices shifted on the fly), so admitting or evicting a
// request costs no host work proportional to the other requests' sizes.
// ---------------------------------------------------------------------------
namespace {

struct src_mesh {
  fvh_mesh_view v;
  int32_t c0, f0, v0, cf0, nb0, cv0;   // destination offsets
  int32_t ncf, nnb, ncv;               // storage lengths
  int32_t keep_from;                   // old first cell of a carried state, or -1
};

constexpr int kGatherThreads = 256, kGatherPerBlock = 256 * 16;

// grid: x = problem, y = chunk of kGatherPerBlock elements
__global__ void gather_cells(const src_mesh *src, fvh_mesh_view dst, int32_t *cell_problem,
                             int dim) {
  const src_mesh &s = src[blockIdx.x];
  const int n = s.v.num_cells;
  for (int i = blockIdx.y * kGatherPerBlock + threadIdx.x;
       i < n && i < (int)(blockIdx.y + 1) * kGatherPerBlock; i += kGatherThreads) {
    const int g = s.c0 + i;
    cell_problem[g] = blockIdx.x;
    const_cast<int32_t *>(dst.cell_face_offsets)[g] = s.v.cell_face_offsets[i] + s.cf0;
    const_cast<int32_t *>(dst.cell_nbr_offsets)[g] = s.v.cell_nbr_offsets[i] + s.nb0;
    const_cast<int32_t *>(dst.cell_vertex_offsets)[g] = s.v.cell_vertex_offsets[i] + s.cv0;
    for (int d = 0; d < dim; ++d) const_cast<double *>(dst.cell_centroid[d])[g] = s.v.cell_centroid[d][i];
    const_cast<double *>(dst.cell_volume)[g] = s.v.cell_volume[i];
  }
}

__global__ void gather_faces(const src_mesh *src, fvh_mesh_view dst, int dim) {
  const src_mesh &s = src[blockIdx.x];
  const int n = s.v.num_faces;
  for (int i = blockIdx.y * kGatherPerBlock + threadIdx.x;
       i < n && i < (int)(blockIdx.y + 1) * kGatherPerBlock; i += kGatherThreads) {
    const int g = s.f0 + i;
    const int a = s.v.face_cells[2 * (size_t)i], b = s.v.face_cells[2 * (size_t)i + 1];
    int32_t *fc = const_cast<int32_t *>(dst.face_cells);
    fc[2 * (size_t)g] = a + s.c0;
    fc[2 * (size_t)g + 1] = b < 0 ? -1 : b + s.c0;
    for (int d = 0; d < dim; ++d) {
      const_cast<double *>(dst.face_centroid[d])[g] = s.v.face_centroid[d][i];
      const_cast<double *>(dst.face_normal[d])[g] = s.v.face_normal[d][i];
    }
    const_cast<double *>(dst.face_area)[g] = s.v.face_area[i];
  }
}

__global__ void gather_vertices(const src_mesh *src, fvh_mesh_view dst, int dim) {
  const src_mesh &s = src[blockIdx.x];
  const int n = s.v.num_vertices;
  for (int i = blockIdx.y * kGatherPerBlock + threadIdx.x;
       i < n && i < (int)(blockIdx.y + 1) * kGatherPerBlock; i += kGatherThreads)
    for (int d = 0; d < dim; ++d)
      const_cast<double *>(dst.vertex_coord[d])[s.v0 + i] = s.v.vertex_coord[d][i];
}

// which = 0: cell_faces (signed face ids), 1: cell_nbrs, 2: cell_vertices
__global__ void gather_csr(const src_mesh *src, fvh_mesh_view dst, int which) {
  const src_mesh &s = src[blockIdx.x];
  const int n = which == 0 ? s.ncf : which == 1 ? s.nnb : s.ncv;
  const int32_t *in = which == 0 ? s.v.cell_faces : which == 1 ? s.v.cell_nbrs : s.v.cell_vertices;
  int32_t *out = const_cast<int32_t *>(which == 0 ? dst.cell_faces
                                       : which == 1 ? dst.cell_nbrs : dst.cell_vertices);
  const int o = which == 0 ? s.cf0 : which == 1 ? s.nb0 : s.cv0;
  for (int i = blockIdx.y * kGatherPerBlock + threadIdx.x;
       i < n && i < (int)(blockIdx.y + 1) * kGatherPerBlock; i += kGatherThreads) {
    const int x = in[i];
    out[o + i] = which == 0 ? (x >= 0 ? x + s.f0 : ~(~x + s.f0)) : which == 1 ? x + s.c0 : x + s.v0;
  }
}

// carried states: new buffer <- old buffer, per problem with keep_from >= 0
__global__ void gather_state(const src_mesh *src, const double *old_buf, double *new_buf,
                             int64_t stride, int planes) {
  const src_mesh &s = src[blockIdx.x];
  if (s.keep_from < 0) return;
  const int n = s.v.num_cells;
  for (int i = blockIdx.y * kGatherPerBlock + threadIdx.x;
       i < n && i < (int)(blockIdx.y + 1) * kGatherPerBlock; i += kGatherThreads)
    for (int pl = 0; pl < planes; ++pl)
      new_buf[pl * stride + s.c0 + i] = old_buf[pl * stride + s.keep_from + i];
}

}  // namespace

fvh_status fvh_batch_assign_device(fvh_batch *b, int32_t n,
                                   const fvh_device_mesh *const *meshes, const double *cfl,
                                   const double *final_time, const int32_t *keep,
                                   fvh_stream_t stream) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!b || n <= 0 || !meshes || !cfl || !final_time) return FVH_ERR_INVALID_ARGUMENT;
    if (n > b->max_problems) return FVH_ERR_CAPACITY;
    const int D = b->dim;
    std::vector<src_mesh> src(n);
    int64_t nc = 0, nf = 0, nv = 0, ncf = 0, nnb = 0, ncv = 0;
    int maxc = 0, maxf = 0, maxv = 0, maxcsr = 0;
    for (int k = 0; k < n; ++k) {
      const fvh_device_mesh *m = meshes[k];
      if (!m || m->view.dim != D || !(cfl[k] > 0)) return FVH_ERR_INVALID_ARGUMENT;
      if (keep && keep[k] >= b->nproblems) return FVH_ERR_INVALID_ARGUMENT;
      src_mesh &s = src[k];
      s.v = m->view;
      s.c0 = (int32_t)nc; s.f0 = (int32_t)nf; s.v0 = (int32_t)nv;
      s.cf0 = (int32_t)ncf; s.nb0 = (int32_t)nnb; s.cv0 = (int32_t)ncv;
      s.ncf = m->nnz_cf; s.nnb = m->nnz_nb; s.ncv = m->nnz_cv;
      s.keep_from = -1;
      if (keep && keep[k] >= 0) {
        const int o = keep[k];
        if (b->first_cell[o + 1] - b->first_cell[o] != m->view.num_cells) return FVH_ERR_INVALID_ARGUMENT;
        s.keep_from = b->first_cell[o];
      }
      nc += m->view.num_cells; nf += m->view.num_faces; nv += m->view.num_vertices;
      ncf += m->nnz_cf; nnb += m->nnz_nb; ncv += m->nnz_cv;
      maxc = std::max(maxc, m->view.num_cells);
      maxf = std::max(maxf, m->view.num_faces);
      maxv = std::max(maxv, m->view.num_vertices);
      maxcsr = std::max({maxcsr, m->nnz_cf, m->nnz_nb, m->nnz_cv});
    }
    if (nc > b->max_cells || nf > b->max_faces || nv > b->max_vertices || ncf > b->max_cf ||
        nnb > b->max_nb || ncv > b->max_cv)
      return FVH_ERR_CAPACITY;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    std::vector<double> times(n, 0.0);
    if (keep && b->nproblems > 0) {
      e = cudaMemcpyAsync(b->h_t, b->t, sizeof(double) * b->nproblems, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      for (int k = 0; k < n; ++k)
        if (keep[k] >= 0) times[k] = b->h_t[keep[k]];
    }
    // destination view, committed to the batch only once everything succeeded
    fvh_mesh_view v;
    std::memset(&v, 0, sizeof(v));
    v.dim = D;
    v.num_cells = (int32_t)nc;
    v.num_faces = (int32_t)nf;
    v.num_vertices = (int32_t)nv;
    v.face_cells = b->face_cells;
    v.cell_face_offsets = b->cf_off;
    v.cell_faces = b->cf;
    v.cell_nbr_offsets = b->nb_off;
    v.cell_nbrs = b->nb;
    v.cell_vertex_offsets = b->cv_off;
    v.cell_vertices = b->cv;
    double *g = b->geo;
    for (int d = 0; d < D; ++d, g += b->max_cells) v.cell_centroid[d] = g;
    v.cell_volume = g;
    g += b->max_cells;
    for (int d = 0; d < D; ++d, g += b->max_faces) v.face_centroid[d] = g;
    for (int d = 0; d < D; ++d, g += b->max_faces) v.face_normal[d] = g;
    v.face_area = g;
    g += b->max_faces;
    for (int d = 0; d < D; ++d, g += b->max_vertices) v.vertex_coord[d] = g;
    // descriptors (device copy), problem tables
    std::vector<int32_t> first(n + 1);
    for (int k = 0; k < n; ++k) first[k] = src[k].c0;
    first[n] = (int32_t)nc;
    src_mesh *d_src = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync(&d_src, sizeof(src_mesh) * n, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_src, src.data(), sizeof(src_mesh) * n, cudaMemcpyHostToDevice, st);
    const int32_t tails[3] = {(int32_t)ncf, (int32_t)nnb, (int32_t)ncv};
    int32_t *tail_dst[3] = {b->cf_off + nc, b->nb_off + nc, b->cv_off + nc};
    for (int q = 0; q < 3 && e == cudaSuccess; ++q)
      e = cudaMemcpyAsync(tail_dst[q], &tails[q], sizeof(int32_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b->d_first_cell, first.data(), sizeof(int32_t) * (n + 1),
                          cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->cfl, cfl, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b->tf, final_time, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->t, times.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dtinv_bits, 0, sizeof(unsigned) * n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->status, 0xff, sizeof(fvh_device_status) * n, st);
    const int nxt = 1 - b->cur;
    if (e == cudaSuccess) {
      auto chunks = [](int m) { return std::max(1, (m + kGatherPerBlock - 1) / kGatherPerBlock); };
      gather_cells<<<dim3(n, chunks(maxc)), kGatherThreads, 0, st>>>(d_src, v, b->cell_problem, D);
      gather_faces<<<dim3(n, chunks(maxf)), kGatherThreads, 0, st>>>(d_src, v, D);
      gather_vertices<<<dim3(n, chunks(maxv)), kGatherThreads, 0, st>>>(d_src, v, D);
      for (int which = 0; which < 3; ++which)
        gather_csr<<<dim3(n, chunks(maxcsr)), kGatherThreads, 0, st>>>(d_src, v, which);
      gather_state<<<dim3(n, chunks(maxc)), kGatherThreads, 0, st>>>(
          d_src, b->state_buf[b->cur], b->state_buf[nxt], b->max_cells, 5 + D);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = fvh::mixed::setup_geometry(b->ws, v, st);
    if (d_src) cudaFreeAsync(d_src, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_assign(b, e);
    b->view = v;
    b->cur = nxt;
    set_state_view(b);
    b->first_cell = std::move(first);
    b->nproblems = n;
    drop_graphs(b);
    return FVH_OK;
  });
}

fvh_status fvh_batch_set_state(fvh_batch *b, int32_t k, const double *host_planes, double t,
                               fvh_stream_t stream) {
  if (!b || k < 0 || k >= b->nproblems || !host_planes) return FVH_ERR_INVALID_ARGUMENT;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int64_t nc = b->first_cell[k + 1] - b->first_cell[k], stride = b->max_cells;
  cudaError_t e = cudaSuccess;
  for (int pl = 0; pl < 5 + b->dim && e == cudaSuccess; ++pl)
    e = cudaMemcpyAsync(b->state_buf[b->cur] + pl * stride + b->first_cell[k],
                        host_planes + pl * nc, sizeof(double) * nc, cudaMemcpyHostToDevice, st);
  b->h_t[k] = t;
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->t + k, b->h_t + k, sizeof(double), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->status + k, 0xff, sizeof(fvh_device_status), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return from_cuda(e);
}

fvh_status fvh_batch_get_state(fvh_batch *b, int32_t k, double *host_planes, fvh_stream_t stream) {
  if (!b || k < 0 || k >= b->nproblems || !host_planes) return FVH_ERR_INVALID_ARGUMENT;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int64_t nc = b->first_cell[k + 1] - b->first_cell[k], stride = b->max_cells;
  cudaError_t e = cudaSuccess;
  for (int pl = 0; pl < 5 + b->dim && e == cudaSuccess; ++pl)
    e = cudaMemcpyAsync(host_planes + pl * nc, b->state_buf[b->cur] + pl * stride + b->first_cell[k],
                        sizeof(double) * nc, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return from_cuda(e);
}

fvh_status fvh_batch_set_shape(fvh_batch *b, int32_t block, int32_t cells_per_thread,
                               int32_t schedule) {
  if (!b || !batch_shape_ok(block, cells_per_thread, schedule)) return FVH_ERR_INVALID_ARGUMENT;
  b->shape.block = block;
  b->shape.cells_per_thread = cells_per_thread;
  b->shape.schedule = schedule;
  drop_graphs(b);
  return FVH_OK;
}

fvh_status fvh_batch_step(fvh_batch *b, int32_t nsteps, fvh_stream_t stream) {
  if (!b || nsteps <= 0 || b->nproblems <= 0) return FVH_ERR_INVALID_ARGUMENT;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const fvh::mixed::problem_map pm = pmap(b);
  // within one call the state is the batch's own: each corrector but the
  // last prepares the next step's pack and per-problem CFL maxima
  auto flags = [nsteps](int k) {
    fvh::mixed::step_flags f;
    f.pack_first = k == 0;
    f.write_next = k + 1 < nsteps;
    return f;
  };
  if (!st) {
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < nsteps && e == cudaSuccess; ++k)
      e = fvh::mixed::step_batch(b->ws, b->view, b->params, b->state, pm, b->shape, st, {},
                                 flags(k));
    return from_cuda(e);
  }
  if (b->graph_stream != st) {
    drop_graphs(b);
    b->graph_stream = st;
  }
  auto it = b->graphs.find(nsteps);
  if (it == b->graphs.end()) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return from_cuda(e);
    cudaError_t le = cudaSuccess;
    for (int k = 0; k < nsteps && le == cudaSuccess; ++k)
      le = fvh::mixed::step_batch(b->ws, b->view, b->params, b->state, pm, b->shape, st, {},
                                  flags(k));
    e = cudaStreamEndCapture(st, &g);
    if (le != cudaSuccess || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return from_cuda(le != cudaSuccess ? le : e);
    }
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return from_cuda(e);
    try {  // no exception crosses the C ABI
      it = b->graphs.emplace(nsteps, ex).first;
    } catch (const std::bad_alloc &) {
      cudaGraphExecDestroy(ex);
      return FVH_ERR_OUT_OF_MEMORY;
    }
  }
  return from_cuda(cudaGraphLaunch(it->second, st));
}

fvh_status fvh_batch_query(fvh_batch *b, double *times, int32_t *codes, int64_t *bad_cells,
                           fvh_stream_t stream) {
  if (!b) return FVH_ERR_INVALID_ARGUMENT;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int n = b->nproblems;
  cudaError_t e = cudaMemcpyAsync(b->h_t, b->t, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->h_status, b->status, sizeof(fvh_device_status) * n,
                        cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return from_cuda(e);
  fvh_status worst = FVH_OK;
  for (int k = 0; k < n; ++k) {
    int32_t code;
    int64_t cell;
    fvh_status_decode(b->h_status[k], &code, &cell);
    if (cell >= 0) cell -= b->first_cell[k];  // cell id within the problem
    if (times) times[k] = b->h_t[k];
    if (codes) codes[k] = code;
    if (bad_cells) bad_cells[k] = cell;
    if (code != FVH_OK && worst == FVH_OK) worst = (fvh_status)code;
  }
  return worst;
}

// ---------------------------------------------------------------------------
// autotuner: time each launch shape on the live batch, keep the fastest
// ---------------------------------------------------------------------------
namespace {

std::string tune_key(const fvh_batch *b) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, dev);
  const int64_t nc = b->view.num_cells;
  int bucket = 0;
  while ((int64_t(1) << (bucket + 1)) <= nc) ++bucket;
  char buf[512];
  std::snprintf(buf, sizeof buf, "%s|sm%d|d%d|f%d|l%d|o%d|c2^%d|p%d", prop.name,
                prop.multiProcessorCount, b->dim, b->params.flux_kind, b->params.limiter,
                b->params.order, bucket, b->nproblems > 1 ? 1 : 0);
  for (char *c = buf; *c; ++c)
    if (*c == ' ' || *c == '\n') *c = '_';
  return buf;
}

std::string cache_path() {
  if (const char *p = std::getenv("FVH_AUTOTUNE_CACHE")) return p;
  const char *home = std::getenv("HOME");
  return std::string(home ? home : ".") + "/.cache/flecsale_gb300_autotune.txt";
}

bool cache_lookup(const std::string &key, fvh::mixed::launch_shape *sh) {
  std::FILE *f = std::fopen(cache_path().c_str(), "r");
  if (!f) return false;
  char line[768];
  bool found = false;
  while (std::fgets(line, sizeof line, f)) {
    char k[512];
    int blk, cpt, sch;
    if (std::sscanf(line, "%511s %d %d %d", k, &blk, &cpt, &sch) == 4 && key == k &&
        batch_shape_ok(blk, cpt, sch)) {
      sh->block = blk;
      sh->cells_per_thread = cpt;
      sh->schedule = sch;
      found = true;  // the last entry for a key wins
    }
  }
  std::fclose(f);
  return found;
}

void cache_store(const std::string &key, const fvh::mixed::launch_shape &sh, double ms) {
  std::FILE *f = std::fopen(cache_path().c_str(), "a");
  if (!f) return;
  std::fprintf(f, "%s %d %d %d %.6f\n", key.c_str(), sh.block, sh.cells_per_thread, sh.schedule,
               ms);
  std::fclose(f);
}

}  // namespace

fvh_status fvh_batch_autotune(fvh_batch *b, int32_t trial_steps, int32_t use_cache,
                              int32_t *block, int32_t *cells_per_thread, int32_t *schedule,
                              double *best_ms_per_step, fvh_stream_t stream) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!b || b->nproblems <= 0 || trial_steps <= 0) return FVH_ERR_INVALID_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const std::string key = tune_key(b);
    fvh::mixed::launch_shape best = b->shape;
    double best_ms = -1.0;
    if (use_cache && cache_lookup(key, &best)) {
      b->shape = best;
      drop_graphs(b);
    } else {
      // save everything a step changes: state planes, times, status words
      const int D = b->dim, P = b->nproblems;
      const int64_t nc = b->view.num_cells, stride = b->max_cells;
      double *saved = nullptr;
      cudaError_t e = cudaMalloc(&saved, sizeof(double) * ((5 + D) * nc + 2 * (size_t)P));
      if (e != cudaSuccess) return from_cuda(e);
      auto copy_state = [&](bool save) {
        for (int pl = 0; pl < 5 + D && e == cudaSuccess; ++pl) {
          double *live = b->state_buf[b->cur] + pl * stride, *bak = saved + pl * nc;
          e = cudaMemcpyAsync(save ? bak : live, save ? live : bak, sizeof(double) * nc,
                              cudaMemcpyDeviceToDevice, st);
        }
        double *bak_t = saved + (5 + D) * nc, *bak_s = bak_t + P;
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(save ? bak_t : b->t, save ? b->t : bak_t, sizeof(double) * P,
                              cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(save ? (void *)bak_s : (void *)b->status,
                              save ? (const void *)b->status : (const void *)bak_s,
                              sizeof(fvh_device_status) * P, cudaMemcpyDeviceToDevice, st);
      };
      copy_state(true);
      const auto &cands = fvh::mixed::kShapes;
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      // every shape timed in each of kAutotuneRounds interleaved rounds; a
      // shape's figure is its fastest round
      constexpr int NS = fvh::mixed::kNumShapes;
      double shape_ms[NS];
      for (int i = 0; i < NS; ++i) shape_ms[i] = -1;
      for (int round = 0; round < fvh::mixed::kAutotuneRounds; ++round) {
        for (int i = 0; i < NS; ++i) {
          const auto &c = cands[i];
          if (e != cudaSuccess) break;
          if (c.schedule == 2) continue;  // the batch has no face colouring
          b->shape = c;
          drop_graphs(b);
          copy_state(false);
          fvh_status r = fvh_batch_step(b, trial_steps, stream);  // capture + warm-up
          if (r == FVH_OK) {
            copy_state(false);
            cudaEventRecord(e0, st);
            r = fvh_batch_step(b, trial_steps, stream);
            cudaEventRecord(e1, st);
          }
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
          best = cands[i];
        }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      copy_state(false);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      cudaFree(saved);
      if (e != cudaSuccess) return from_cuda(e);
      b->shape = best;
      drop_graphs(b);
      if (best_ms > 0) cache_store(key, best, best_ms);
    }
    if (block) *block = best.block;
    if (cells_per_thread) *cells_per_thread = best.cells_per_thread;
    if (schedule) *schedule = best.schedule;
    if (best_ms_per_step) *best_ms_per_step = best_ms;
    return FVH_OK;
  });
}

int32_t fvh_batch_num_problems(const fvh_batch *b) { return b ? b->nproblems : 0; }
int64_t fvh_batch_num_cells(const fvh_batch *b) { return b ? b->view.num_cells : 0; }
int32_t fvh_batch_launches_per_step(const fvh_batch *b) {
  if (!b) return 0;
  fvh::mixed::step_flags f;  // a step after the first of a call
  f.pack_first = false;
  f.write_next = true;
  return fvh::mixed::launches_per_step_batch(b->params, b->shape, f);
}

}  // extern "C"
