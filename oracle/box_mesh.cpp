// ORACLE — test infrastructure only.
//
// A structured 2D box of quads built independently of the product's mesh
// builder, so the CPU baseline of the benchmark and the tests can set up the
// benchmark workload without loading the product library.  The result is
// meant to be identical, array for array and bit for bit, to the product's
// general builder on the same box (tests/test_oracle_box_mesh.py checks that).
//
// The reference takes its mesh from the flecsi-sp "burton" specialization,
// whose sources are absent from the reference tree; the queries the hydro
// tasks make of it are listed at apps/hydro/tasks.h:170-273 (centroid, volume,
// face area/normal/centroid, cells(f), faces(c), vertices(c),
// cell_vertex_neighbors(c)).  The rules fixed here, for a box of nx x ny quads:
//   * vertex (i, j) has id i + (nx+1) j; interior vertices are jittered by
//     jitter*h*(2u-1) per axis, u the SplitMix64 uniform of stream
//     (seed, 3 v + axis) (Steele, Lea & Flood 2014);
//   * cell (i, j) has id i + nx j and vertices (i,j) (i+1,j) (i+1,j+1) (i,j+1);
//     its local face k is the edge from vertex k to vertex k+1;
//   * faces get ids in order of first encounter, walking cells by id and each
//     cell's local faces in order; a face belongs to the lower cell id, whose
//     local edge gives the face's vertex order and its outward normal;
//   * cell_vertex_neighbors(c) are the (up to 8) cells sharing a vertex with c,
//     in ascending id;
//   * geometry: shoelace area and centroid of each quad; face centroid at the
//     edge midpoint, area = edge length, normal = (dy, -dx) / length.
#include <cmath>
#include <cstdint>

#include <omp.h>

namespace {

uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

double uniform01(uint64_t seed, uint64_t counter) {
  const uint64_t z = splitmix64(splitmix64(seed) ^ (counter * 0xD1B54A32D192ED03ull));
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// faces created by cell (i, j): bottom (j == 0), right, top, left (i == 0)
inline int64_t faces_before_cell(int64_t nx, int64_t i, int64_t j) {
  // row j: every cell creates right + top; the row-0 cells also bottom; the
  // column-0 cell also left
  const int64_t per_row = 2 * nx + 1;  // + the left face of cell (0, j)
  const int64_t before_rows = j * per_row + (j > 0 ? nx : 0);
  const int64_t in_row = 2 * i + (j == 0 ? i : 0) + (i > 0 ? 1 : 0);
  return before_rows + in_row;
}

}  // namespace

extern "C" {

// Sizes of the nx x ny box: vertices, faces, cell->face and cell->neighbour
// list lengths.
void oracle_box2d_sizes(int32_t nx, int32_t ny, int64_t *nv, int64_t *nf,
                        int64_t *ncf, int64_t *nnb) {
  const int64_t X = nx, Y = ny;
  *nv = (X + 1) * (Y + 1);
  *nf = X * (Y + 1) + (X + 1) * Y;
  *ncf = 4 * X * Y;
  // 8 neighbours per cell, minus those outside the box
  const int64_t nbx = (X == 1) ? 0 : 2 * (X - 1);  // horizontal adjacencies x2
  const int64_t nby = (Y == 1) ? 0 : 2 * (Y - 1);
  *nnb = nbx * Y + nby * X + 4 * (X - 1) * (Y - 1);
}

// Fills caller-allocated arrays (sizes from oracle_box2d_sizes).  Geometry
// planes are SoA: vertex_coord[2][nv], cell_centroid[2][nc], face_centroid and
// face_normal [2][nf].
void oracle_box2d_build(int32_t nx, int32_t ny, double x0, double y0, double x1, double y1,
                        double jitter, uint64_t seed,
                        int32_t *face_cells, int32_t *cell_face_offsets, int32_t *cell_faces,
                        int32_t *cell_nbr_offsets, int32_t *cell_nbrs,
                        int32_t *cell_vertex_offsets, int32_t *cell_vertices,
                        double *cell_centroid, double *cell_volume, double *face_centroid,
                        double *face_normal, double *face_area, double *vertex_coord) {
  const int64_t X = nx, Y = ny, nvx = X + 1, nvy = Y + 1, nc = X * Y;
  const int64_t nv = nvx * nvy;
  const int64_t nf = X * (Y + 1) + (X + 1) * Y;
  const double lo[2] = {x0, y0}, hi[2] = {x1, y1};
  const double h[2] = {(x1 - x0) / nx, (y1 - y0) / ny};
  double *vx = vertex_coord, *vy = vertex_coord + nv;
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < nv; ++v) {
    const int64_t idx[2] = {v % nvx, v / nvx};
    const int64_t nvd[2] = {nvx, nvy};
    bool boundary = false;
    for (int d = 0; d < 2; ++d)
      if (idx[d] == 0 || idx[d] == nvd[d] - 1) boundary = true;
    for (int d = 0; d < 2; ++d) {
      double x = idx[d] == nvd[d] - 1 ? hi[d] : lo[d] + (double)idx[d] * h[d];
      if (!boundary && jitter > 0)
        x += (2.0 * uniform01(seed, (uint64_t)v * 3 + d) - 1.0) * jitter * h[d];
      (d == 0 ? vx : vy)[v] = x;
    }
  }
  auto vid = [&](int64_t i, int64_t j) { return (int32_t)(i + nvx * j); };
  auto cid = [&](int64_t i, int64_t j) { return (int32_t)(i + X * j); };
  // per cell: its 4 local faces' ids (creator's id for shared faces)
  auto face_id = [&](int64_t i, int64_t j, int k) -> int64_t {
    // ids of the faces created by (i, j), in creation order
    const int64_t base = faces_before_cell(X, i, j);
    const int64_t bottom = base;                           // only if j == 0
    const int64_t right = base + (j == 0 ? 1 : 0);
    const int64_t top = right + 1;
    const int64_t left = top + 1;                          // only if i == 0
    switch (k) {
      case 0: return j == 0 ? bottom : faces_before_cell(X, i, j - 1) + (j - 1 == 0 ? 1 : 0) + 1;
      case 1: return right;
      case 2: return top;
      default: return i == 0 ? left : faces_before_cell(X, i - 1, j) + (j == 0 ? 1 : 0);
    }
  };
  double *ccx = cell_centroid, *ccy = cell_centroid + nc;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    const int64_t i = c % X, j = c / X;
    const int32_t v4[4] = {vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)};
    cell_vertex_offsets[c] = (int32_t)(4 * c);
    cell_face_offsets[c] = (int32_t)(4 * c);
    for (int k = 0; k < 4; ++k) cell_vertices[4 * c + k] = v4[k];
    // faces(c) with orientation: created here -> f, else ~f
    const bool created[4] = {j == 0, true, true, i == 0};
    for (int k = 0; k < 4; ++k) {
      const int32_t f = (int32_t)face_id(i, j, k);
      cell_faces[4 * c + k] = created[k] ? f : ~f;
    }
    // creator side of each created face: cells(f) = (c, neighbour or -1)
    const int32_t nbr[4] = {j > 0 ? cid(i, j - 1) : -1, i + 1 < X ? cid(i + 1, j) : -1,
                            j + 1 < Y ? cid(i, j + 1) : -1, i > 0 ? cid(i - 1, j) : -1};
    for (int k = 0; k < 4; ++k)
      if (created[k]) {
        const int32_t f = cell_faces[4 * c + k];
        face_cells[2 * (int64_t)f] = (int32_t)c;
        face_cells[2 * (int64_t)f + 1] = nbr[k];
        // edge k = (v_k, v_k+1): midpoint, length, normal (dy, -dx) / length
        const int32_t a = v4[k], b = v4[(k + 1) % 4];
        const double xa = vx[a], ya = vy[a], xb = vx[b], yb = vy[b];
        const double dx = xb - xa, dy = yb - ya;
        const double len = std::sqrt(dx * dx + dy * dy);
        face_centroid[f] = 0.5 * (xa + xb);
        face_centroid[nf + f] = 0.5 * (ya + yb);
        face_area[f] = len;
        face_normal[f] = dy / len;
        face_normal[nf + f] = -dx / len;
      }
    // shoelace area and area-weighted centroid, vertices in order
    double a2 = 0, sx = 0, sy = 0;
    for (int k = 0; k < 4; ++k) {
      const int32_t p = v4[k], q = v4[(k + 1) % 4];
      const double xp = vx[p], yp = vy[p], xq = vx[q], yq = vy[q];
      const double cr = xp * yq - xq * yp;
      a2 += cr;
      sx += (xp + xq) * cr;
      sy += (yp + yq) * cr;
    }
    cell_volume[c] = 0.5 * a2;
    ccx[c] = sx / (3.0 * a2);
    ccy[c] = sy / (3.0 * a2);
  }
  cell_vertex_offsets[nc] = (int32_t)(4 * nc);
  cell_face_offsets[nc] = (int32_t)(4 * nc);
  // vertex neighbours, ascending id: rows j-1, j, j+1; columns i-1, i, i+1
  auto count_nb = [&](int64_t i, int64_t j) {
    const int64_t ci = 1 + (i > 0) + (i + 1 < X), cj = 1 + (j > 0) + (j + 1 < Y);
    return ci * cj - 1;
  };
  // offsets by rows: every row has the same counts pattern except the ends
  int64_t acc = 0;
  for (int64_t c = 0; c < nc; ++c) {
    cell_nbr_offsets[c] = (int32_t)acc;
    acc += count_nb(c % X, c / X);
  }
  cell_nbr_offsets[nc] = (int32_t)acc;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    const int64_t i = c % X, j = c / X;
    int32_t *o = cell_nbrs + cell_nbr_offsets[c];
    for (int64_t jj = j - 1; jj <= j + 1; ++jj)
      for (int64_t ii = i - 1; ii <= i + 1; ++ii) {
        if (ii < 0 || jj < 0 || ii >= X || jj >= Y || (ii == i && jj == j)) continue;
        *o++ = cid(ii, jj);
      }
  }
}

}  // extern "C"
