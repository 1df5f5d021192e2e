// Input files of apps/hydro: the Lua "hydro" table read by
// apps/hydro/inputs.h:100-135 (prefix, postfix, output_freq, CFL, final_time,
// max_steps, eos = {type, gas_constant, specific_heat}, ics = function), plus
// the box mesh table of apps/hydro/3d/shock_box_3d.lua.  Evaluated with the
// Lua-subset interpreter of fvh_lua.cpp.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "flecsale_gb300.h"
#include "fvh_internal.h"
#include "fvh_lua.h"

using fvh::lua::Value;

struct fvh_input {
  fvh::lua::State state;
};

namespace {

void set_err(char *err, size_t len, const std::string &m) {
  if (!err || len == 0) return;
  const size_t n = m.size() < len - 1 ? m.size() : len - 1;
  std::memcpy(err, m.data(), n);
  err[n] = '\0';
}

Value at(const fvh_input *in, const std::string &path) {
  const size_t dot = path.find_first_of(".[");
  const std::string head = path.substr(0, dot);
  const Value g = in->state.global(head);
  return dot == std::string::npos ? g : fvh::lua::lookup(g, path.substr(dot));
}

bool as_number(const Value &v, double *out) {
  if (v.kind == Value::NUMBER) {
    *out = v.n;
    return true;
  }
  if (v.kind == Value::STRING) {  // "1e6": Lua converts numeric strings
    char *e = nullptr;
    const double d = std::strtod(v.s.c_str(), &e);
    if (e != v.s.c_str() && *e == '\0') {
      *out = d;
      return true;
    }
  }
  return false;
}

fvh_status load(const std::string &text, const std::string &name, char *err, size_t err_len,
                fvh_input **out) {
  fvh_input *in = new (std::nothrow) fvh_input();
  if (!in) return FVH_ERR_OUT_OF_MEMORY;
  try {
    in->state.run(text, name);
  } catch (const std::exception &e) {
    set_err(err, err_len, e.what());
    delete in;
    return FVH_ERR_INVALID_ARGUMENT;
  }
  if (in->state.global("hydro").kind != Value::TABLE) {
    set_err(err, err_len, name + ": no table 'hydro'");
    delete in;
    return FVH_ERR_INVALID_ARGUMENT;
  }
  *out = in;
  return FVH_OK;
}

}  // namespace

extern "C" {

fvh_status fvh_input_load(const char *path, char *err, size_t err_len, fvh_input **out) {
  if (!path || !out) return FVH_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    set_err(err, err_len, std::string("cannot open ") + path);
    return FVH_ERR_INVALID_ARGUMENT;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  // the chunk name Lua would report: the file name
  std::string name = path;
  const size_t slash = name.find_last_of('/');
  if (slash != std::string::npos) name = name.substr(slash + 1);
  return load(ss.str(), name, err, err_len, out);
}

fvh_status fvh_input_load_string(const char *text, char *err, size_t err_len, fvh_input **out) {
  if (!text || !out) return FVH_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  return load(text, "input", err, err_len, out);
}

void fvh_input_destroy(fvh_input *in) { delete in; }

fvh_status fvh_input_number(const fvh_input *in, const char *path, double *value) {
  if (!in || !path || !value) return FVH_ERR_INVALID_ARGUMENT;
  return as_number(at(in, path), value) ? FVH_OK : FVH_ERR_INVALID_ARGUMENT;
}

fvh_status fvh_input_string(const fvh_input *in, const char *path, char *buf, size_t len) {
  if (!in || !path || !buf || len == 0) return FVH_ERR_INVALID_ARGUMENT;
  const Value v = at(in, path);
  if (v.kind != Value::STRING) return FVH_ERR_INVALID_ARGUMENT;
  if (v.s.size() + 1 > len) return FVH_ERR_CAPACITY;
  std::memcpy(buf, v.s.c_str(), v.s.size() + 1);
  return FVH_OK;
}

fvh_status fvh_input_params(const fvh_input *in, fvh_params *p, int64_t *max_steps,
                            int64_t *output_freq) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!in || !p) return FVH_ERR_INVALID_ARGUMENT;
    // values are checked before they are stored: counts are whole and
    // non-negative (they convert to int64 exactly), CFL and the EOS constants
    // positive and finite (gamma > 1), the final time not NaN
    double v;
    auto count = [&](const char *key, int64_t *out) -> bool {
      if (!out || !as_number(at(in, key), &v)) return true;
      if (!(v >= 0 && v <= 9.0e18) || v != std::floor(v)) return false;
      *out = (int64_t)v;
      return true;
    };
    fvh_params q = *p;
    if (as_number(at(in, "hydro.CFL"), &v)) q.cfl = v;
    if (as_number(at(in, "hydro.final_time"), &v)) q.final_time = v;
    const Value eos = at(in, "hydro.eos");
    if (eos.kind == Value::TABLE) {
      const Value type = fvh::lua::lookup(eos, "type");
      if (type.kind != Value::STRING || type.s != "ideal_gas")
        return FVH_ERR_UNSUPPORTED;  // inputs.h:129-131 "Unknown eos type"
      if (as_number(fvh::lua::lookup(eos, "gas_constant"), &v)) q.gamma = v;
      if (as_number(fvh::lua::lookup(eos, "specific_heat"), &v)) q.cv = v;
    }
    if (!(q.cfl > 0) || !std::isfinite(q.cfl) || std::isnan(q.final_time) || !(q.gamma > 1) ||
        !std::isfinite(q.gamma) || !(q.cv > 0) || !std::isfinite(q.cv))
      return FVH_ERR_INVALID_ARGUMENT;
    int64_t ms = max_steps ? *max_steps : 0, of = output_freq ? *output_freq : 0;
    if (!count("hydro.max_steps", max_steps ? &ms : nullptr) ||
        !count("hydro.output_freq", output_freq ? &of : nullptr))
      return FVH_ERR_INVALID_ARGUMENT;
    *p = q;
    if (max_steps) *max_steps = ms;
    if (output_freq) *output_freq = of;
    return FVH_OK;
  });
}

fvh_status fvh_input_mesh(const fvh_input *in, fvh_host_mesh **out) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!in || !out) return FVH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    const Value mesh = at(in, "hydro.mesh");
    if (mesh.kind != Value::TABLE) return FVH_ERR_INVALID_ARGUMENT;
    const Value type = fvh::lua::lookup(mesh, "type");
    if (type.kind != Value::STRING || type.s != "box") return FVH_ERR_UNSUPPORTED;
    const Value dims = fvh::lua::lookup(mesh, "dimensions");
    if (dims.kind != Value::TABLE) return FVH_ERR_INVALID_ARGUMENT;
    const int dim = (int)dims.t->array.size();
    if (dim != 2 && dim != 3) return FVH_ERR_INVALID_ARGUMENT;
    int32_t n[3];
    double lo[3], hi[3];
    for (int k = 0; k < dim; ++k) {
      double v;
      const std::string idx = "[" + std::to_string(k + 1) + "]";
      // a whole number of cells that int32 holds (NaN and fractions refused)
      if (!as_number(dims.t->array[k], &v) || !(v >= 1 && v <= 2147483647.0) ||
          v != std::floor(v))
        return FVH_ERR_INVALID_ARGUMENT;
      n[k] = (int32_t)v;
      lo[k] = 0;
      hi[k] = 1;
      if (as_number(fvh::lua::lookup(mesh, "xmin" + idx), &v)) lo[k] = v;
      if (as_number(fvh::lua::lookup(mesh, "xmax" + idx), &v)) hi[k] = v;
    }
    return fvh_host_mesh_box(dim, n, lo, hi, 0.0, 0, out);
  });
}

fvh_status fvh_input_initial_state(const fvh_input *in, const fvh_host_mesh *m,
                                   const fvh_params *p, double t, double *host_planes) {
  return fvh::no_throw([&]() -> fvh_status {
    if (!in || !m || !p || !host_planes || p->dim != m->dim) return FVH_ERR_INVALID_ARGUMENT;
    const Value ics = at(in, "hydro.ics");
    if (ics.kind != Value::FUNCTION) return FVH_ERR_INVALID_ARGUMENT;
    const int D = m->dim, nc = m->nc;
    std::vector<double> d(nc), v((size_t)D * nc), pr(nc);
    fvh::lua::State &st = const_cast<fvh_input *>(in)->state;
    try {
      std::vector<Value> args(D + 1);
      for (int c = 0; c < nc; ++c) {
        for (int k = 0; k < D; ++k) args[k] = Value::number(m->cc[k][c]);
        args[D] = Value::number(t);
        const std::vector<Value> r = st.call(ics, args);
        // initial_conditions (tasks.h:46-68): density, velocity, pressure
        if (r.size() < 3 || r[0].kind != Value::NUMBER || r[1].kind != Value::TABLE ||
            r[2].kind != Value::NUMBER)
          return FVH_ERR_INVALID_ARGUMENT;
        d[c] = r[0].n;
        pr[c] = r[2].n;
        // positive, finite density and pressure (the reference asserts both,
        // euler_eqns.h:342-343) and finite velocity
        if (!(d[c] > 0) || !(pr[c] > 0) || !std::isfinite(d[c]) || !std::isfinite(pr[c]))
          return FVH_ERR_INVALID_ARGUMENT;
        for (int k = 0; k < D; ++k) {
          const Value vk = r[1].t->get(Value::number(k + 1));
          v[(size_t)k * nc + c] = vk.kind == Value::NUMBER ? vk.n : 0.0;
          if (!std::isfinite(v[(size_t)k * nc + c])) return FVH_ERR_INVALID_ARGUMENT;
        }
      }
    } catch (const std::bad_alloc &) {
      throw;  // FVH_ERR_OUT_OF_MEMORY
    } catch (const std::exception &) {
      return FVH_ERR_INVALID_ARGUMENT;
    }
    return fvh_host_state_from_dvp(D, nc, p->gamma, p->cv, d.data(), v.data(), pr.data(),
                                   host_planes);
  });
}

}  // extern "C"
