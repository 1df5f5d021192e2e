// Host-side mesh topology and geometry for the finite-volume hydro step.
//
// The reference takes these from the flecsi-sp "burton" mesh specialization
// (apps/hydro/types.h:33), whose sources are not part of the reference tree.
// The hydro tasks use only these queries of it:
//   cells(f), faces(c)            tasks.h:414,479,629,632
//   cell_vertex_neighbors(c)      tasks.h:190
//   vertices(c)                   tasks.h:270
//   c->centroid(), c->volume()    tasks.h:170,196,357,419,644
//   f->centroid(), f->area(), f->normal()   tasks.h:357,359,411,453,461
//   v->coordinates()              tasks.h:273
// This file builds all of them from cell -> vertex lists, with the rules
// written next to each routine.  Ordering rules (they fix the floating-point
// summation order of the kernels):
//   * faces get ids in order of first encounter while walking cells by id and
//     each cell's local faces in order; cells(f)[0] is the cell that created the
//     face (the lower id), and the face normal points out of it;
//   * faces(c) is the cell's local face order (polygon edge k = (v_k, v_k+1);
//     Exodus side order for hexahedra and tetrahedra);
//   * cell_vertex_neighbors(c) is the set of cells sharing a vertex with c,
//     excluding c, in ascending cell id.
#include "flecsale_gb300.h"
#include "fvh_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

namespace {

// Exodus side numbering (outward normals by the right-hand rule).
const int kHexFaces[6][4] = {{0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6},
                             {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};
const int kTetFaces[4][3] = {{0, 1, 3}, {1, 2, 3}, {0, 3, 2}, {0, 2, 1}};

// Local faces of one cell as vertex lists (global ids).
struct local_faces {
  int n = 0;            // number of faces
  int nv[6] = {0};      // vertices per face (2D: 2)
  int v[6][4] = {{0}};
};

// Polygons with more than 6 edges are split into repeated calls by index.
inline int polygon_edge(const int32_t *cv, int nverts, int k, int *out) {
  out[0] = cv[k];
  out[1] = cv[(k + 1) % nverts];
  return 2;
}

bool cell_faces_of(int dim, const int32_t *cv, int nverts, int k, int *out,
                   int *nout) {
  if (dim == 2) {
    *nout = polygon_edge(cv, nverts, k, out);
    return true;
  }
  if (nverts == 8) {
    for (int i = 0; i < 4; ++i) out[i] = cv[kHexFaces[k][i]];
    *nout = 4;
    return true;
  }
  if (nverts == 4) {
    for (int i = 0; i < 3; ++i) out[i] = cv[kTetFaces[k][i]];
    *nout = 3;
    return true;
  }
  return false;
}

int num_local_faces(int dim, int nverts) {
  if (dim == 2) return nverts >= 3 ? nverts : -1;
  if (nverts == 8) return 6;
  if (nverts == 4) return 4;
  return -1;
}

// true when every vertex of the face (fv, nfv) is a vertex of cell c
bool cell_has_all(const fvh_host_mesh &m, int c, const int *fv, int nfv) {
  const int32_t *b = m.cv.data() + m.cv_off[c];
  const int32_t *e = m.cv.data() + m.cv_off[c + 1];
  for (int i = 0; i < nfv; ++i)
    if (std::find(b, e, fv[i]) == e) return false;
  return true;
}

}  // namespace

namespace fvh {

// Geometry of one 2D polygon (shoelace area and area-weighted centroid).
static void polygon_geometry(const fvh_host_mesh &m, int c, double *cx,
                             double *cy, double *area) {
  const int b = m.cv_off[c], n = m.cv_off[c + 1] - b;
  double a2 = 0, sx = 0, sy = 0;
  for (int k = 0; k < n; ++k) {
    const int v0 = m.cv[b + k], v1 = m.cv[b + (k + 1) % n];
    const double x0 = m.vc[0][v0], y0 = m.vc[1][v0];
    const double x1 = m.vc[0][v1], y1 = m.vc[1][v1];
    const double cr = x0 * y1 - x1 * y0;
    a2 += cr;
    sx += (x0 + x1) * cr;
    sy += (y0 + y1) * cr;
  }
  *area = 0.5 * a2;
  *cx = sx / (3.0 * a2);
  *cy = sy / (3.0 * a2);
}

// Geometry of one 3D face given its vertex list in outward order: the face is
// fanned into triangles about the vertex average xm; the area vector is the sum
// of the triangle area vectors, the centroid the triangle-area-weighted mean of
// the triangle centroids.
static void face3_geometry(const fvh_host_mesh &m, const int *fv, int n,
                           double sv[3], double cen[3]) {
  double xm[3] = {0, 0, 0};
  for (int k = 0; k < n; ++k)
    for (int d = 0; d < 3; ++d) xm[d] += m.vc[d][fv[k]];
  for (int d = 0; d < 3; ++d) xm[d] /= n;
  sv[0] = sv[1] = sv[2] = 0;
  double wsum = 0, ws[3] = {0, 0, 0};
  for (int k = 0; k < n; ++k) {
    const int a = fv[k], b = fv[(k + 1) % n];
    double ea[3], eb[3];
    for (int d = 0; d < 3; ++d) {
      ea[d] = m.vc[d][a] - xm[d];
      eb[d] = m.vc[d][b] - xm[d];
    }
    const double t[3] = {0.5 * (ea[1] * eb[2] - ea[2] * eb[1]),
                         0.5 * (ea[2] * eb[0] - ea[0] * eb[2]),
                         0.5 * (ea[0] * eb[1] - ea[1] * eb[0])};
    const double w = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    for (int d = 0; d < 3; ++d) {
      sv[d] += t[d];
      ws[d] += w * (xm[d] + m.vc[d][a] + m.vc[d][b]) / 3.0;
    }
    wsum += w;
  }
  for (int d = 0; d < 3; ++d) cen[d] = wsum > 0 ? ws[d] / wsum : xm[d];
}

// Volume and centroid of a 3D cell: tetrahedra (cell vertex average, face
// vertex average, edge) over the triangulated faces, in outward orientation.
static void cell3_geometry(const fvh_host_mesh &m, int c, double cen[3],
                           double *vol) {
  const int b = m.cv_off[c], nv = m.cv_off[c + 1] - b;
  const int32_t *cv = m.cv.data() + b;
  double xc[3] = {0, 0, 0};
  for (int k = 0; k < nv; ++k)
    for (int d = 0; d < 3; ++d) xc[d] += m.vc[d][cv[k]];
  for (int d = 0; d < 3; ++d) xc[d] /= nv;
  const int nlf = num_local_faces(3, nv);
  double v = 0, s[3] = {0, 0, 0};
  for (int lf = 0; lf < nlf; ++lf) {
    int fv[4], nfv;
    cell_faces_of(3, cv, nv, lf, fv, &nfv);
    double xm[3] = {0, 0, 0};
    for (int k = 0; k < nfv; ++k)
      for (int d = 0; d < 3; ++d) xm[d] += m.vc[d][fv[k]];
    for (int d = 0; d < 3; ++d) xm[d] /= nfv;
    for (int k = 0; k < nfv; ++k) {
      const int a = fv[k], bb = fv[(k + 1) % nfv];
      double p[3], q[3], r[3];
      for (int d = 0; d < 3; ++d) {
        p[d] = xm[d] - xc[d];
        q[d] = m.vc[d][a] - xc[d];
        r[d] = m.vc[d][bb] - xc[d];
      }
      // signed volume of (xc, xm, a, b); positive for outward (a, b) order
      const double t = (q[0] * (r[1] * p[2] - r[2] * p[1]) +
                        q[1] * (r[2] * p[0] - r[0] * p[2]) +
                        q[2] * (r[0] * p[1] - r[1] * p[0])) /
                       6.0;
      v += t;
      for (int d = 0; d < 3; ++d)
        s[d] += t * (xc[d] + xm[d] + m.vc[d][a] + m.vc[d][bb]) / 4.0;
    }
  }
  *vol = v;
  for (int d = 0; d < 3; ++d) cen[d] = v != 0 ? s[d] / v : xc[d];
}

fvh_status build_topology_and_geometry(fvh_host_mesh &m) {
  const int dim = m.dim, nc = m.nc, nv = m.nv;
  // vertex -> cells, ascending cell id
  std::vector<int32_t> vc_off(nv + 1, 0), vcl;
  for (int c = 0; c < nc; ++c) {
    for (int k = m.cv_off[c]; k < m.cv_off[c + 1]; ++k) {
      const int v = m.cv[k];
      if (v < 0 || v >= nv) return FVH_ERR_INVALID_ARGUMENT;
      // a vertex listed twice makes a degenerate face that would match a
      // neighbour sharing that vertex
      for (int j = m.cv_off[c]; j < k; ++j)
        if (m.cv[j] == v) return FVH_ERR_INVALID_ARGUMENT;
      vc_off[v + 1]++;
    }
  }
  for (int v = 0; v < nv; ++v) vc_off[v + 1] += vc_off[v];
  vcl.resize(vc_off[nv]);
  {
    std::vector<int32_t> fill(vc_off.begin(), vc_off.end() - 1);
    for (int c = 0; c < nc; ++c)
      for (int k = m.cv_off[c]; k < m.cv_off[c + 1]; ++k)
        vcl[fill[m.cv[k]]++] = c;
  }

  // local faces and their neighbour across each one
  std::vector<int32_t> lf_off(nc + 1, 0);
  for (int c = 0; c < nc; ++c) {
    const int n = num_local_faces(dim, m.cv_off[c + 1] - m.cv_off[c]);
    if (n < 0) return FVH_ERR_UNSUPPORTED;
    lf_off[c + 1] = lf_off[c] + n;
  }
  const int64_t nlf = lf_off[nc];
  std::vector<int32_t> lf_nbr(nlf, -1);
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int c = 0; c < nc; ++c) {
    const int32_t *cv = m.cv.data() + m.cv_off[c];
    const int ncv = m.cv_off[c + 1] - m.cv_off[c];
    for (int k = 0; k < lf_off[c + 1] - lf_off[c]; ++k) {
      int fv[4], nfv;
      cell_faces_of(dim, cv, ncv, k, fv, &nfv);
      int found = -1, count = 0;
      for (int q = vc_off[fv[0]]; q < vc_off[fv[0] + 1]; ++q) {
        const int c1 = vcl[q];
        if (c1 == c) continue;
        if (cell_has_all(m, c1, fv, nfv)) {
          found = c1;
          ++count;
        }
      }
      if (count > 1) bad = 1;
      lf_nbr[lf_off[c] + k] = found;
    }
    // two faces of one cell shared with the same neighbour: not supported
    for (int64_t q = lf_off[c]; q < lf_off[c + 1]; ++q)
      for (int64_t r = lf_off[c]; r < q; ++r)
        if (lf_nbr[q] >= 0 && lf_nbr[q] == lf_nbr[r]) bad = 1;
  }
  if (bad) return FVH_ERR_UNSUPPORTED;  // non-manifold face

  // face ids in order of first encounter
  std::vector<int32_t> lf_face(nlf, -1);
  int32_t nf = 0;
  for (int c = 0; c < nc; ++c)
    for (int64_t q = lf_off[c]; q < lf_off[c + 1]; ++q)
      if (lf_nbr[q] < 0 || lf_nbr[q] > c) lf_face[q] = nf++;
  m.nf = nf;
  m.face_cells.assign(2 * (size_t)nf, -1);
  m.fv_off.assign(nf + 1, 0);
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int c = 0; c < nc; ++c)
    for (int64_t q = lf_off[c]; q < lf_off[c + 1]; ++q) {
      const int nb = lf_nbr[q];
      if (nb >= 0 && nb < c) {
        // created by nb: find nb's local face that points back at c
        int hit = -1;
        for (int64_t r = lf_off[nb]; r < lf_off[nb + 1]; ++r)
          if (lf_nbr[r] == c) {
            if (hit >= 0) bad = 1;  // two shared faces: not supported
            hit = lf_face[r];
          }
        if (hit < 0) bad = 1;
        lf_face[q] = hit;
      } else {
        m.face_cells[2 * (size_t)lf_face[q]] = c;
        m.face_cells[2 * (size_t)lf_face[q] + 1] = nb;
      }
    }
  if (bad) return FVH_ERR_UNSUPPORTED;

  // faces(c), signed by orientation
  m.cf_off.assign(lf_off.begin(), lf_off.end());
  m.cf.resize(nlf);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c)
    for (int64_t q = lf_off[c]; q < lf_off[c + 1]; ++q) {
      const int f = lf_face[q];
      m.cf[q] = (m.face_cells[2 * (size_t)f] == c) ? f : ~f;
    }

  // every interior face is listed by its second cell too (as ~f), exactly once:
  // otherwise its flux would leave one cell and enter none
  {
    std::vector<int32_t> second(nf, -1);
    for (int c = 0; c < nc && !bad; ++c)
      for (int64_t q = lf_off[c]; q < lf_off[c + 1]; ++q)
        if (m.cf[q] < 0) {
          const int f = ~m.cf[q];
          if (second[f] >= 0 || m.face_cells[2 * (size_t)f + 1] != c) bad = 1;
          second[f] = c;
        }
    for (int f = 0; f < nf && !bad; ++f)
      if ((m.face_cells[2 * (size_t)f + 1] >= 0) != (second[f] >= 0)) bad = 1;
    if (bad) return FVH_ERR_UNSUPPORTED;
  }

  // face -> vertices (creator's orientation)
  std::vector<int> fnv(nf, 0);
  for (int c = 0; c < nc; ++c) {
    const int32_t *cv = m.cv.data() + m.cv_off[c];
    const int ncv = m.cv_off[c + 1] - m.cv_off[c];
    for (int64_t q = lf_off[c]; q < lf_off[c + 1]; ++q)
      if (m.cf[q] >= 0) {
        int fv[4], n;
        cell_faces_of(dim, cv, ncv, (int)(q - lf_off[c]), fv, &n);
        fnv[m.cf[q]] = n;
      }
  }
  for (int f = 0; f < nf; ++f) m.fv_off[f + 1] = m.fv_off[f] + fnv[f];
  m.fv.resize(m.fv_off[nf]);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    const int32_t *cv = m.cv.data() + m.cv_off[c];
    const int ncv = m.cv_off[c + 1] - m.cv_off[c];
    for (int64_t q = lf_off[c]; q < lf_off[c + 1]; ++q)
      if (m.cf[q] >= 0) {
        int fv[4], n;
        cell_faces_of(dim, cv, ncv, (int)(q - lf_off[c]), fv, &n);
        for (int i = 0; i < n; ++i) m.fv[m.fv_off[m.cf[q]] + i] = fv[i];
      }
  }

  // cell_vertex_neighbors(c): cells sharing a vertex, ascending id
  std::vector<int32_t> nbcount(nc + 1, 0);
  std::vector<std::vector<int32_t>> nbl(nc);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    std::vector<int32_t> &l = nbl[c];
    for (int k = m.cv_off[c]; k < m.cv_off[c + 1]; ++k) {
      const int v = m.cv[k];
      for (int q = vc_off[v]; q < vc_off[v + 1]; ++q)
        if (vcl[q] != c) l.push_back(vcl[q]);
    }
    std::sort(l.begin(), l.end());
    l.erase(std::unique(l.begin(), l.end()), l.end());
    nbcount[c + 1] = (int32_t)l.size();
  }
  m.nb_off.assign(nc + 1, 0);
  for (int c = 0; c < nc; ++c) m.nb_off[c + 1] = m.nb_off[c] + nbcount[c + 1];
  m.nb.resize(m.nb_off[nc]);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nc; ++c) {
    std::copy(nbl[c].begin(), nbl[c].end(), m.nb.begin() + m.nb_off[c]);
    std::vector<int32_t>().swap(nbl[c]);
  }

  // geometry
  for (int d = 0; d < 3; ++d) {
    m.cc[d].assign(d < dim ? nc : 0, 0.0);
    m.fc[d].assign(d < dim ? nf : 0, 0.0);
    m.fn[d].assign(d < dim ? nf : 0, 0.0);
  }
  m.cvol.assign(nc, 0.0);
  m.fa.assign(nf, 0.0);
  if (dim == 2) {
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nc; ++c)
      polygon_geometry(m, c, &m.cc[0][c], &m.cc[1][c], &m.cvol[c]);
#pragma omp parallel for schedule(static)
    for (int f = 0; f < nf; ++f) {
      const int a = m.fv[m.fv_off[f]], b = m.fv[m.fv_off[f] + 1];
      const double xa = m.vc[0][a], ya = m.vc[1][a];
      const double xb = m.vc[0][b], yb = m.vc[1][b];
      const double dx = xb - xa, dy = yb - ya;
      const double len = std::sqrt(dx * dx + dy * dy);
      m.fc[0][f] = 0.5 * (xa + xb);
      m.fc[1][f] = 0.5 * (ya + yb);
      m.fa[f] = len;
      m.fn[0][f] = dy / len;
      m.fn[1][f] = -dx / len;
    }
  } else {
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nc; ++c) {
      double cen[3];
      cell3_geometry(m, c, cen, &m.cvol[c]);
      for (int d = 0; d < 3; ++d) m.cc[d][c] = cen[d];
    }
#pragma omp parallel for schedule(static)
    for (int f = 0; f < nf; ++f) {
      double sv[3], cen[3];
      face3_geometry(m, m.fv.data() + m.fv_off[f], m.fv_off[f + 1] - m.fv_off[f],
                     sv, cen);
      const double a = std::sqrt(sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2]);
      m.fa[f] = a;
      for (int d = 0; d < 3; ++d) {
        m.fn[d][f] = sv[d] / a;
        m.fc[d][f] = cen[d];
      }
    }
  }
  for (int c = 0; c < nc; ++c)
    if (!(m.cvol[c] > 0)) return FVH_ERR_INVALID_ARGUMENT;  // inverted cell
  for (int f = 0; f < nf; ++f)
    if (!(m.fa[f] > 0)) return FVH_ERR_INVALID_ARGUMENT;    // face of zero extent
  // every cell is closed: the sum of its outward area vectors vanishes (to
  // rounding), so a uniform state is a steady state of the update
  for (int c = 0; c < nc; ++c) {
    double sum[3] = {0, 0, 0}, area = 0;
    for (int64_t q = m.cf_off[c]; q < m.cf_off[c + 1]; ++q) {
      const int32_t e = m.cf[q];
      const int f = e >= 0 ? e : ~e;
      const double sgn = e >= 0 ? 1.0 : -1.0;
      for (int d = 0; d < dim; ++d) sum[d] += sgn * m.fa[f] * m.fn[d][f];
      area += m.fa[f];
    }
    const double gap = std::sqrt(sum[0] * sum[0] + sum[1] * sum[1] + sum[2] * sum[2]);
    if (!(gap <= 1e-10 * area)) return FVH_ERR_INVALID_ARGUMENT;
  }
  return FVH_OK;
}

// SplitMix64 (Steele, Lea & Flood 2014): one 64-bit output per counter value.
static inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Uniform double in [0, 1) for stream (seed, counter).
double uniform01(uint64_t seed, uint64_t counter) {
  const uint64_t z = splitmix64(splitmix64(seed) ^ (counter * 0xD1B54A32D192ED03ull));
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace fvh

extern "C" {

fvh_status fvh_host_mesh_create(int32_t dim, int32_t num_vertices,
                                const double *vertex_coords, int32_t num_cells,
                                const int32_t *cell_vertex_offsets,
                                const int32_t *cell_vertices,
                                fvh_host_mesh **out) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!out || (dim != 2 && dim != 3) || num_vertices <= 0 || num_cells <= 0 ||
        !vertex_coords || !cell_vertex_offsets || !cell_vertices)
      return FVH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::unique_ptr<fvh_host_mesh> m(new (std::nothrow) fvh_host_mesh());
    if (!m) return FVH_ERR_OUT_OF_MEMORY;
    m->dim = dim;
    m->nv = num_vertices;
    m->nc = num_cells;
    for (int d = 0; d < 3; ++d) m->vc[d].assign(d < dim ? num_vertices : 0, 0.0);
    for (int v = 0; v < num_vertices; ++v)
      for (int d = 0; d < dim; ++d) m->vc[d][v] = vertex_coords[(size_t)v * dim + d];
    m->cv_off.assign(cell_vertex_offsets, cell_vertex_offsets + num_cells + 1);
    if (m->cv_off[0] != 0) return FVH_ERR_INVALID_ARGUMENT;
    for (int c = 0; c < num_cells; ++c)
      if (m->cv_off[c + 1] <= m->cv_off[c]) return FVH_ERR_INVALID_ARGUMENT;
    m->cv.assign(cell_vertices, cell_vertices + m->cv_off[num_cells]);
    const fvh_status st = fvh::build_topology_and_geometry(*m);
    if (st != FVH_OK) return st;
    *out = m.release();
    return FVH_OK;
  });
}

fvh_status fvh_host_mesh_box(int32_t dim, const int32_t *n, const double *lo,
                             const double *hi, double jitter, uint64_t seed,
                             fvh_host_mesh **out) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!out || !n || !lo || !hi || (dim != 2 && dim != 3) || !(jitter >= 0 && jitter < 0.5))
      return FVH_ERR_INVALID_ARGUMENT;
    int64_t nvx[3] = {1, 1, 1}, ncx[3] = {1, 1, 1};
    double h[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      if (n[d] <= 0 || !(hi[d] > lo[d]) || !std::isfinite(lo[d]) || !std::isfinite(hi[d]))
        return FVH_ERR_INVALID_ARGUMENT;
      ncx[d] = n[d];
      nvx[d] = n[d] + 1;
      h[d] = (hi[d] - lo[d]) / n[d];
    }
    const int64_t nv = nvx[0] * nvx[1] * nvx[2];
    const int64_t nc = ncx[0] * ncx[1] * ncx[2];
    if (nv >= INT32_MAX || nc * (dim == 2 ? 4 : 8) >= INT32_MAX)
      return FVH_ERR_CAPACITY;
    std::vector<double> xyz((size_t)nv * dim);
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < nv; ++v) {
      const int64_t idx[3] = {v % nvx[0], (v / nvx[0]) % nvx[1], v / (nvx[0] * nvx[1])};
      bool boundary = false;
      for (int d = 0; d < dim; ++d)
        if (idx[d] == 0 || idx[d] == nvx[d] - 1) boundary = true;
      for (int d = 0; d < dim; ++d) {
        double x = idx[d] == nvx[d] - 1 ? hi[d] : lo[d] + (double)idx[d] * h[d];
        if (!boundary && jitter > 0)
          x += (2.0 * fvh::uniform01(seed, (uint64_t)v * 3 + d) - 1.0) * jitter * h[d];
        xyz[(size_t)v * dim + d] = x;
      }
    }
    const int per = dim == 2 ? 4 : 8;
    std::vector<int32_t> off((size_t)nc + 1), cv((size_t)nc * per);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nc; ++c) {
      const int64_t i = c % ncx[0], j = (c / ncx[0]) % ncx[1], k = c / (ncx[0] * ncx[1]);
      auto vid = [&](int64_t a, int64_t b, int64_t cc) {
        return (int32_t)(a + nvx[0] * (b + nvx[1] * cc));
      };
      int32_t *o = cv.data() + c * per;
      o[0] = vid(i, j, k);
      o[1] = vid(i + 1, j, k);
      o[2] = vid(i + 1, j + 1, k);
      o[3] = vid(i, j + 1, k);
      if (dim == 3) {
        o[4] = vid(i, j, k + 1);
        o[5] = vid(i + 1, j, k + 1);
        o[6] = vid(i + 1, j + 1, k + 1);
        o[7] = vid(i, j + 1, k + 1);
      }
      off[c] = (int32_t)(c * per);
    }
    off[nc] = (int32_t)(nc * per);
    return fvh_host_mesh_create(dim, (int32_t)nv, xyz.data(), (int32_t)nc,
                                off.data(), cv.data(), out);
  });
}

void fvh_host_mesh_destroy(fvh_host_mesh *m) { delete m; }

fvh_status fvh_host_mesh_concat(int32_t n, const fvh_host_mesh *const *meshes,
                                fvh_host_mesh **out) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!out || n <= 0 || !meshes) return FVH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    const int dim = meshes[0] ? meshes[0]->dim : 0;
    int64_t nc = 0, nf = 0, nv = 0, ncf = 0, nnb = 0, ncv = 0, nfv = 0;
    for (int k = 0; k < n; ++k) {
      const fvh_host_mesh *m = meshes[k];
      if (!m || m->dim != dim) return FVH_ERR_INVALID_ARGUMENT;
      nc += m->nc; nf += m->nf; nv += m->nv;
      ncf += m->cf.size(); nnb += m->nb.size(); ncv += m->cv.size(); nfv += m->fv.size();
    }
    if (nc >= INT32_MAX || nf >= INT32_MAX || nv >= INT32_MAX || ncf >= INT32_MAX ||
        nnb >= INT32_MAX || ncv >= INT32_MAX || nfv >= INT32_MAX)
      return FVH_ERR_CAPACITY;
    std::unique_ptr<fvh_host_mesh> o(new (std::nothrow) fvh_host_mesh());
    if (!o) return FVH_ERR_OUT_OF_MEMORY;
    o->dim = dim;
    o->nc = (int)nc; o->nf = (int)nf; o->nv = (int)nv;
    o->cf_off.assign(1, 0); o->nb_off.assign(1, 0); o->cv_off.assign(1, 0); o->fv_off.assign(1, 0);
    int32_t co = 0, fo = 0, vo = 0;
    for (int k = 0; k < n; ++k) {
      const fvh_host_mesh &m = *meshes[k];
      for (int f = 0; f < m.nf; ++f) {
        const int32_t a = m.face_cells[2 * (size_t)f], b = m.face_cells[2 * (size_t)f + 1];
        o->face_cells.push_back(a + co);
        o->face_cells.push_back(b < 0 ? -1 : b + co);
      }
      auto append_csr = [](std::vector<int32_t> &off, std::vector<int32_t> &dst,
                           const std::vector<int32_t> &soff, const std::vector<int32_t> &src,
                           auto shift) {
        const int32_t base = off.back();
        for (size_t i = 1; i < soff.size(); ++i) off.push_back(base + soff[i]);
        for (int32_t x : src) dst.push_back(shift(x));
      };
      append_csr(o->cf_off, o->cf, m.cf_off, m.cf, [fo](int32_t f) { return f >= 0 ? f + fo : ~(~f + fo); });
      append_csr(o->nb_off, o->nb, m.nb_off, m.nb, [co](int32_t c) { return c + co; });
      append_csr(o->cv_off, o->cv, m.cv_off, m.cv, [vo](int32_t v) { return v + vo; });
      append_csr(o->fv_off, o->fv, m.fv_off, m.fv, [vo](int32_t v) { return v + vo; });
      for (int d = 0; d < 3; ++d) {
        o->cc[d].insert(o->cc[d].end(), m.cc[d].begin(), m.cc[d].end());
        o->fc[d].insert(o->fc[d].end(), m.fc[d].begin(), m.fc[d].end());
        o->fn[d].insert(o->fn[d].end(), m.fn[d].begin(), m.fn[d].end());
        o->vc[d].insert(o->vc[d].end(), m.vc[d].begin(), m.vc[d].end());
      }
      o->cvol.insert(o->cvol.end(), m.cvol.begin(), m.cvol.end());
      o->fa.insert(o->fa.end(), m.fa.begin(), m.fa.end());
      co += m.nc; fo += m.nf; vo += m.nv;
    }
    *out = o.release();
    return FVH_OK;
  });
}

fvh_status fvh_host_mesh_view(const fvh_host_mesh *m, fvh_mesh_view *o) {
  if (!m || !o) return FVH_ERR_INVALID_ARGUMENT;
  std::memset(o, 0, sizeof(*o));
  o->dim = m->dim;
  o->num_cells = m->nc;
  o->num_faces = m->nf;
  o->num_vertices = m->nv;
  o->face_cells = m->face_cells.data();
  o->cell_face_offsets = m->cf_off.data();
  o->cell_faces = m->cf.data();
  o->cell_nbr_offsets = m->nb_off.data();
  o->cell_nbrs = m->nb.data();
  o->cell_vertex_offsets = m->cv_off.data();
  o->cell_vertices = m->cv.data();
  for (int d = 0; d < m->dim; ++d) {
    o->cell_centroid[d] = m->cc[d].data();
    o->face_centroid[d] = m->fc[d].data();
    o->face_normal[d] = m->fn[d].data();
    o->vertex_coord[d] = m->vc[d].data();
  }
  o->cell_volume = m->cvol.data();
  o->face_area = m->fa.data();
  return FVH_OK;
}

fvh_status fvh_host_mesh_nnz(const fvh_host_mesh *m, int64_t *cf, int64_t *nb,
                             int64_t *cv) {
  if (!m) return FVH_ERR_INVALID_ARGUMENT;
  if (cf) *cf = (int64_t)m->cf.size();
  if (nb) *nb = (int64_t)m->nb.size();
  if (cv) *cv = (int64_t)m->cv.size();
  return FVH_OK;
}

}  // extern "C"
