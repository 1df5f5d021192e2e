// Internal declarations shared by the library's translation units.
#pragma once

#include <cstdint>
#include <new>
#include <vector>

#include "flecsale_gb300.h"

// Host mesh: topology and geometry arrays (see fvh_mesh.cpp for the rules).
struct fvh_host_mesh {
  int dim = 0, nc = 0, nf = 0, nv = 0;
  std::vector<int32_t> face_cells;          // 2 per face
  std::vector<int32_t> cf_off, cf;          // faces(c), signed
  std::vector<int32_t> nb_off, nb;          // cell_vertex_neighbors(c)
  std::vector<int32_t> cv_off, cv;          // vertices(c)
  std::vector<int32_t> fv_off, fv;          // face -> vertices
  std::vector<double> cc[3], cvol;          // cell centroid, volume
  std::vector<double> fc[3], fn[3], fa;     // face centroid, normal, area
  std::vector<double> vc[3];                // vertex coordinates
};

// Device copy of a host mesh (fvh_device_mesh_create).
struct fvh_device_mesh {
  fvh_mesh_view view{};
  int32_t nnz_cf = 0, nnz_nb = 0, nnz_cv = 0;  // CSR storage lengths
  std::vector<void *> allocs;
};

namespace fvh {
fvh_status build_topology_and_geometry(fvh_host_mesh &m);

// Runs the body of a C entry point so that no C++ exception crosses the C ABI:
// a failed host allocation (std::bad_alloc) becomes FVH_ERR_OUT_OF_MEMORY and
// any other exception FVH_ERR_INVALID_ARGUMENT.  Objects the body builds are
// owned by RAII guards until it succeeds, so an exception leaks nothing.
template <class Body>
fvh_status no_throw(Body &&body) noexcept {
  try {
    return body();
  } catch (const std::bad_alloc &) {
    return FVH_ERR_OUT_OF_MEMORY;
  } catch (...) {
    return FVH_ERR_INVALID_ARGUMENT;
  }
}

double uniform01(uint64_t seed, uint64_t counter);
}  // namespace fvh
