// Host IO around the hydro step:
//  * the regression dump of apps/hydro/tasks.h:771-849 (the text file the
//    reference's regression tests diff against their .std goldens);
//  * an Exodus II reader for the netCDF classic (CDF-1) and 64-bit-offset
//    (CDF-2) encodings, enough for the reference's meshes in data/meshes
//    (QUAD4 / SHELL4 / HEX8 / TETRA4 blocks; coordinates as coordx/coordy/
//    coordz or as one coord variable).  netCDF-4 (HDF5) files are not read.
//  * the EOS closure for caller-provided (density, velocity, pressure), the
//    second half of initial_conditions (apps/hydro/tasks.h:58-66).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "flecsale_gb300.h"
#include "fvh_internal.h"

namespace {

// ---------------------------------------------------------------------------
// netCDF classic reader (big-endian)
// ---------------------------------------------------------------------------
struct nc_var {
  std::string name;
  std::vector<int> dims;
  int type = 0;
  uint64_t begin = 0, vsize = 0;
  std::vector<std::pair<std::string, std::string>> text_attrs;
};

struct nc_file {
  // netCDF's own limit on the dimensions of one variable (NC_MAX_VAR_DIMS)
  static constexpr uint32_t kMaxVarDims = 1024;
  std::vector<uint8_t> buf;
  size_t pos = 0;
  bool cdf2 = false, bad = false;
  std::vector<std::pair<std::string, uint64_t>> dims;
  std::vector<nc_var> vars;

  uint32_t u32() {
    if (pos + 4 > buf.size()) { bad = true; return 0; }
    const uint32_t v = (uint32_t)buf[pos] << 24 | (uint32_t)buf[pos + 1] << 16 |
                       (uint32_t)buf[pos + 2] << 8 | buf[pos + 3];
    pos += 4;
    return v;
  }
  uint64_t u64() {
    const uint64_t hi = u32();
    return hi << 32 | u32();
  }
  std::string name() {
    const uint32_t n = u32();
    if (bad || pos + n > buf.size()) { bad = true; return {}; }
    std::string s(reinterpret_cast<const char *>(&buf[pos]), n);
    pos += (n + 3) / 4 * 4;
    return s;
  }
  static int type_size(int t) {
    switch (t) {
      case 1: case 2: return 1;
      case 3: return 2;
      case 4: case 5: return 4;
      case 6: return 8;
      default: return 0;
    }
  }
  // attribute list; text attributes are kept
  void attrs(std::vector<std::pair<std::string, std::string>> *keep) {
    const uint32_t tag = u32(), n = u32();
    if (tag == 0 && n == 0) return;
    if (tag != 0x0C) { bad = true; return; }
    for (uint32_t i = 0; i < n && !bad; ++i) {
      const std::string an = name();
      const int t = (int)u32();
      const uint32_t ne = u32();
      const size_t bytes = (size_t)ne * type_size(t);
      if (pos + bytes > buf.size() || type_size(t) == 0) { bad = true; return; }
      if (keep && t == 2)
        keep->emplace_back(an, std::string(reinterpret_cast<const char *>(&buf[pos]), ne));
      pos += (bytes + 3) / 4 * 4;
    }
  }
  bool parse() {
    if (buf.size() < 8 || std::memcmp(buf.data(), "CDF", 3) != 0) return false;
    if (buf[3] != 1 && buf[3] != 2) return false;
    cdf2 = buf[3] == 2;
    pos = 4;
    u32();  // numrecs
    uint32_t tag = u32(), n = u32();
    if (tag == 0x0A) {
      for (uint32_t i = 0; i < n && !bad; ++i) {
        const std::string dn = name();
        dims.emplace_back(dn, u32());
      }
    } else if (!(tag == 0 && n == 0)) {
      return false;
    }
    attrs(nullptr);
    tag = u32();
    n = u32();
    if (tag == 0x0B) {
      for (uint32_t i = 0; i < n && !bad; ++i) {
        nc_var v;
        v.name = name();
        const uint32_t nd = u32();
        // every dimension id must name a dimension of this file
        if (nd > kMaxVarDims) { bad = true; break; }
        for (uint32_t k = 0; k < nd && !bad; ++k) {
          const uint32_t id = u32();
          if (id >= dims.size()) bad = true;
          v.dims.push_back((int)id);
        }
        attrs(&v.text_attrs);
        v.type = (int)u32();
        v.vsize = u32();
        v.begin = cdf2 ? u64() : u32();
        vars.push_back(v);
      }
    }
    return !bad;
  }
  const nc_var *var(const std::string &n) const {
    for (const auto &v : vars)
      if (v.name == n) return &v;
    return nullptr;
  }
  // elements of a variable; UINT64_MAX when the product overflows
  uint64_t count(const nc_var &v) const {
    uint64_t c = 1;
    for (int d : v.dims) {
      const uint64_t n = dims[d].second;
      if (n != 0 && c > UINT64_MAX / n) return UINT64_MAX;
      c *= n;
    }
    return c;
  }
  bool is_record(const nc_var &v) const { return !v.dims.empty() && dims[v.dims[0]].second == 0; }
  // fixed-size numeric variable as doubles
  bool read_f64(const nc_var &v, std::vector<double> *out) const {
    if (is_record(v)) return false;
    const uint64_t n = count(v);
    const int ts = type_size(v.type);
    if (ts == 0 || v.begin > buf.size() || n > (buf.size() - v.begin) / ts) return false;
    out->resize(n);
    const uint8_t *p = buf.data() + v.begin;
    for (uint64_t i = 0; i < n; ++i, p += ts) {
      uint64_t bits = 0;
      for (int b = 0; b < ts; ++b) bits = bits << 8 | p[b];
      double x = 0;
      switch (v.type) {
        case 1: x = (int8_t)bits; break;
        case 3: x = (int16_t)bits; break;
        case 4: x = (int32_t)bits; break;
        case 5: { uint32_t u = (uint32_t)bits; float f; std::memcpy(&f, &u, 4); x = f; break; }
        case 6: std::memcpy(&x, &bits, 8); break;
        default: return false;
      }
      (*out)[i] = x;
    }
    return true;
  }
};

std::string attr(const nc_var &v, const char *n) {
  for (const auto &a : v.text_attrs)
    if (a.first == n) {
      std::string s = a.second;
      while (!s.empty() && (s.back() == '\0' || s.back() == ' ')) s.pop_back();
      for (auto &ch : s) ch = (char)std::toupper((unsigned char)ch);
      return s;
    }
  return {};
}

}  // namespace

extern "C" {

fvh_status fvh_host_mesh_read_exodus(const char *path, fvh_host_mesh **out) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!path || !out) return FVH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::FILE *f = std::fopen(path, "rb");
    if (!f) return FVH_ERR_INVALID_ARGUMENT;
    nc_file nc;
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    nc.buf.resize(size > 0 ? (size_t)size : 0);
    const size_t got = nc.buf.empty() ? 0 : std::fread(nc.buf.data(), 1, nc.buf.size(), f);
    std::fclose(f);
    if (got != nc.buf.size() || !nc.parse()) return FVH_ERR_UNSUPPORTED;  // not CDF-1/2
    // coordinates
    std::vector<double> xyz[3];
    int ncoord = 0;
    const char *cn[3] = {"coordx", "coordy", "coordz"};
    for (int d = 0; d < 3; ++d)
      if (const nc_var *v = nc.var(cn[d])) {
        if (!nc.read_f64(*v, &xyz[d])) return FVH_ERR_UNSUPPORTED;
        ncoord = d + 1;
      }
    if (ncoord == 0) {
      const nc_var *v = nc.var("coord");
      std::vector<double> all;
      if (!v || v->dims.size() != 2 || !nc.read_f64(*v, &all)) return FVH_ERR_UNSUPPORTED;
      ncoord = (int)nc.dims[v->dims[0]].second;
      if (ncoord < 2 || ncoord > 3) return FVH_ERR_UNSUPPORTED;
      const size_t nn = nc.dims[v->dims[1]].second;
      for (int d = 0; d < ncoord; ++d) xyz[d].assign(all.begin() + d * nn, all.begin() + (d + 1) * nn);
    }
    // two or three coordinate arrays, all of one length that int32 ids can index
    if (ncoord < 2) return FVH_ERR_UNSUPPORTED;
    const size_t nv = xyz[0].size();
    if (nv == 0 || nv >= (size_t)INT32_MAX) return FVH_ERR_UNSUPPORTED;
    for (int d = 1; d < ncoord; ++d)
      if (xyz[d].size() != nv) return FVH_ERR_UNSUPPORTED;
    // element blocks connect1, connect2, ...
    std::vector<int32_t> off{0}, cells;
    int shape = 0;  // nodes per element of the first block
    bool shell = false;
    for (int blk = 1;; ++blk) {
      const nc_var *v = nc.var("connect" + std::to_string(blk));
      if (!v) break;
      std::vector<double> c;
      if (v->dims.size() != 2 || !nc.read_f64(*v, &c)) return FVH_ERR_UNSUPPORTED;
      const std::string et = attr(*v, "elem_type");
      const uint64_t npe64 = nc.dims[v->dims[1]].second;
      if (npe64 < 3 || npe64 > 8) return FVH_ERR_UNSUPPORTED;
      const int npe = (int)npe64;
      if (shape == 0) shape = npe;
      if (npe != shape) return FVH_ERR_UNSUPPORTED;  // mixed element shapes
      if (et.rfind("SHELL", 0) == 0) shell = true;
      if (cells.size() + c.size() >= (size_t)INT32_MAX) return FVH_ERR_CAPACITY;
      for (size_t k = 0; k + npe <= c.size(); k += npe) {
        for (int q = 0; q < npe; ++q) {
          // Exodus node ids are 1-based; anything else is a malformed file
          const double id = c[k + q];
          if (!(id >= 1 && id <= (double)nv) || id != std::floor(id))
            return FVH_ERR_INVALID_ARGUMENT;
          cells.push_back((int32_t)id - 1);
        }
        off.push_back((int32_t)cells.size());
      }
    }
    if (cells.empty() || nv == 0) return FVH_ERR_UNSUPPORTED;
    // dimension: QUAD4/SHELL4 with a flat z are 2D polygons
    int dim = ncoord;
    if (shape == 4 && (ncoord == 2 || shell)) {
      dim = 2;
      if (ncoord == 3)
        for (double z : xyz[2])
          if (std::fabs(z - xyz[2][0]) > 0) return FVH_ERR_UNSUPPORTED;  // curved shell
    }
    if (dim == 3 && shape != 8 && shape != 4) return FVH_ERR_UNSUPPORTED;
    std::vector<double> coords(nv * dim);
    for (size_t i = 0; i < nv; ++i)
      for (int d = 0; d < dim; ++d) coords[i * dim + d] = xyz[d][i];
    // 2D polygons must be counter-clockwise; reverse clockwise ones
    if (dim == 2) {
      const size_t ncell = off.size() - 1;
      for (size_t c = 0; c < ncell; ++c) {
        double a2 = 0;
        const int b = off[c], n = off[c + 1] - b;
        for (int k = 0; k < n; ++k) {
          const int p = cells[b + k], q = cells[b + (k + 1) % n];
          a2 += coords[2 * p] * coords[2 * q + 1] - coords[2 * q] * coords[2 * p + 1];
        }
        if (a2 < 0) std::reverse(cells.begin() + b + 1, cells.begin() + b + n);
      }
    }
    return fvh_host_mesh_create(dim, (int32_t)nv, coords.data(), (int32_t)(off.size() - 1),
                                off.data(), cells.data(), out);
  });
}

fvh_status fvh_dump_write(const char *path, const fvh_host_mesh *m, const double *host_planes,
                          double soln_time, int64_t iterations) {
  if (!path || !m || !host_planes) return FVH_ERR_INVALID_ARGUMENT;
  std::FILE *f = std::fopen(path, "w");
  if (!f) return FVH_ERR_INVALID_ARGUMENT;
  const int D = m->dim, nc = m->nc;
  const double *d = host_planes, *e = host_planes + (size_t)(1 + D) * nc, *p = e + nc;
  // layout of apps/hydro/tasks.h:805-845: precision(14), scientific
  std::fprintf(f, "# Solution time: %.14e\n", soln_time);
  std::fprintf(f, "# Number iterations: %lld\n", (long long)iterations);
  std::fprintf(f, "# BEGIN CELLS\n# Total number: %d\n# local_id global_id ", nc);
  for (int k = 0; k < D; ++k) std::fprintf(f, "centroid(%d) ", k);
  std::fprintf(f, "density internal_energy pressure ");
  for (int k = 0; k < D; ++k) std::fprintf(f, "velocity(%d) ", k);
  std::fprintf(f, "\n");
  for (int c = 0; c < nc; ++c) {
    std::fprintf(f, "%d %d ", c, c);
    for (int k = 0; k < D; ++k) std::fprintf(f, "%.14e ", m->cc[k][c]);
    std::fprintf(f, "%.14e %.14e %.14e ", d[c], e[c], p[c]);
    for (int k = 0; k < D; ++k) std::fprintf(f, "%.14e ", host_planes[(size_t)(1 + k) * nc + c]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "# END CELLS\n# BEGIN VERTICES\n# Total number: %d\n# local_id global_id ", m->nv);
  for (int k = 0; k < D; ++k) std::fprintf(f, "coordinate(%d) ", k);
  std::fprintf(f, "\n");
  for (int v = 0; v < m->nv; ++v) {
    std::fprintf(f, "%d %d ", v, v);
    for (int k = 0; k < D; ++k) std::fprintf(f, "%.14e ", m->vc[k][v]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "# END VERTICES\n");
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  return ok ? FVH_OK : FVH_ERR_INVALID_ARGUMENT;
}

fvh_status fvh_dump_read(const char *path, int32_t dim, int32_t num_cells, double gamma,
                         double cv, double *host_planes, double *soln_time,
                         int64_t *iterations) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!path || (dim != 2 && dim != 3) || num_cells <= 0 || !host_planes || !(gamma > 1) ||
        !(cv > 0))
      return FVH_ERR_INVALID_ARGUMENT;
    std::FILE *f = std::fopen(path, "r");
    if (!f) return FVH_ERR_INVALID_ARGUMENT;
    std::string line;
    auto next_line = [&]() -> bool {
      line.clear();
      int ch;
      while ((ch = std::fgetc(f)) != EOF && ch != '\n') line.push_back((char)ch);
      return ch != EOF || !line.empty();
    };
    auto after = [&](const char *prefix) -> const char * {
      const size_t n = std::strlen(prefix);
      return line.compare(0, n, prefix) == 0 ? line.c_str() + n : nullptr;
    };
    // header: "# Solution time: t", "# Number iterations: n", "# BEGIN CELLS",
    // "# Total number: N", then the column-name line (tasks.h:805-820)
    double t = 0;
    long long iters = 0;
    bool have_t = false, have_n = false, in_cells = false;
    int64_t total = -1;
    fvh_status st = FVH_OK;
    while (st == FVH_OK && next_line()) {
      const char *v = nullptr;
      char *end = nullptr;
      if ((v = after("# Solution time:"))) {
        t = std::strtod(v, &end);
        have_t = end != v;
      } else if ((v = after("# Number iterations:"))) {
        iters = std::strtoll(v, &end, 10);
        have_n = end != v;
      } else if (after("# BEGIN CELLS")) {
        in_cells = true;
      } else if (in_cells && (v = after("# Total number:"))) {
        total = std::strtoll(v, &end, 10);
        if (end == v || total != num_cells) st = FVH_ERR_INVALID_ARGUMENT;
        if (st == FVH_OK && !next_line()) st = FVH_ERR_INVALID_ARGUMENT;  // column names
        break;
      }
    }
    if (st == FVH_OK && (!have_t || !have_n || total != num_cells)) st = FVH_ERR_INVALID_ARGUMENT;
    // rows: local_id global_id centroid[dim] density internal_energy pressure velocity[dim]
    const size_t nc = (size_t)num_cells;
    double *d = host_planes, *e = host_planes + (size_t)(1 + dim) * nc, *pr = e + nc, *T = pr + nc,
           *a = T + nc;
    std::vector<char> seen(nc, 0);
    for (size_t row = 0; st == FVH_OK && row < nc; ++row) {
      if (!next_line()) {
        st = FVH_ERR_INVALID_ARGUMENT;
        break;
      }
      const int nv = 2 + dim + 3 + dim;
      double x[2 + 3 + 3 + 3];
      const char *q = line.c_str();
      for (int k = 0; k < nv && st == FVH_OK; ++k) {
        char *end = nullptr;
        x[k] = std::strtod(q, &end);
        if (end == q || !std::isfinite(x[k])) st = FVH_ERR_INVALID_ARGUMENT;
        q = end;
      }
      while (st == FVH_OK && *q != '\0') {  // nothing but blanks after the last column
        if (!std::isspace((unsigned char)*q)) st = FVH_ERR_INVALID_ARGUMENT;
        ++q;
      }
      if (st != FVH_OK) break;
      const double id = x[0];
      if (!(id >= 0 && id < (double)nc) || id != std::floor(id) || seen[(size_t)id]) {
        st = FVH_ERR_INVALID_ARGUMENT;
        break;
      }
      const size_t c = (size_t)id;
      seen[c] = 1;
      const double *w = x + 2 + dim;  // density internal_energy pressure velocity...
      d[c] = w[0];
      e[c] = w[1];
      pr[c] = w[2];
      for (int k = 0; k < dim; ++k) host_planes[(size_t)(1 + k) * nc + c] = w[3 + k];
      // closure from the internal energy (update_state_from_energy, euler_eqns.h:359-375)
      T[c] = w[1] / cv;
      a[c] = std::sqrt(gamma * (gamma - 1.0) * w[1]);
    }
    if (st == FVH_OK && (!next_line() || !after("# END CELLS"))) st = FVH_ERR_INVALID_ARGUMENT;
    std::fclose(f);
    if (st != FVH_OK) return st;
    if (soln_time) *soln_time = t;
    if (iterations) *iterations = (int64_t)iters;
    return FVH_OK;
  });
}

fvh_status fvh_host_state_from_dvp(int32_t dim, int32_t n, double gamma, double cv,
                                   const double *density, const double *velocity,
                                   const double *pressure, double *host_planes) {
  if ((dim != 2 && dim != 3) || n <= 0 || !density || !velocity || !pressure || !host_planes ||
      !(gamma > 1) || !(cv > 0))
    return FVH_ERR_INVALID_ARGUMENT;
  double *e = host_planes + (size_t)(1 + dim) * n, *pr = e + n, *T = pr + n, *a = T + n;
  for (int32_t i = 0; i < n; ++i) {
    host_planes[i] = density[i];
    for (int k = 0; k < dim; ++k) host_planes[(size_t)(1 + k) * n + i] = velocity[(size_t)k * n + i];
    pr[i] = pressure[i];
    const double ie = pressure[i] / (density[i] * (gamma - 1.0));  // ideal_gas.h:178-184
    e[i] = ie;
    T[i] = ie / cv;
    a[i] = std::sqrt(gamma * (gamma - 1.0) * ie);
  }
  return FVH_OK;
}

}  // extern "C"
