// flecsale_hydro: the command-line driver of apps/hydro (driver.h:163-450)
// on the GB300 step.  Same options as apps/common/arguments.h:25-70
// (-f/--input_file, -m/--mesh, -e/--max_entries, -h/--help) plus scheme
// choices the reference makes at compile time (types.h:118-137).  Runs
// max_steps steps (dt clamped to final_time - t, tasks.h:343,373), prints the
// final solution time as print_soln_time does (tasks.h:683-700) and writes the
// regression dump <prefix>-solution_rank000000.txt (driver.h:441-445,
// tasks.h:771-849).
#include <getopt.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "flecsale_gb300.h"

namespace {

void usage(const char *argv0) {
  std::printf(
      "Usage: %s [--input_file INPUT_FILE] [--max_entries MAX_ENTRIES] [--mesh MESH_FILE] "
      "[--help]\n\n"
      "\t--input_file INPUT_FILE:\t Override the input file with INPUT_FILE (Lua).\n"
      "\t--max_entries MAX_ENTRIES:\t Accepted for compatibility; unused.\n"
      "\t--mesh MESH_FILE:\t Override the mesh file with MESH_FILE (Exodus II, CDF-1/2).\n"
      "\t--help:\t Print a help message.\n\n"
      "Scheme (compile-time aliases in the reference, types.h:118-137):\n"
      "\t--flux hlle|rusanov|hllc\t (default hlle)\n"
      "\t--limiter barth_jespersen|none\t (default barth_jespersen)\n"
      "\t--boundary wall|outflow\t (default wall)\n"
      "\t--precision fp64|mixed\t (default fp64, the reference arithmetic)\n"
      "\t--order 1|2\t (default 2)\n"
      "\t--output_dir DIR\t where the solution dump goes (default .)\n",
      argv0);
}

int fail(const char *what, int code) {
  std::fprintf(stderr, "flecsale_hydro: %s: %s\n", what, fvh_status_string(code));
  return 1;
}

}  // namespace

int main(int argc, char **argv) {
  static const struct option long_options[] = {
      {"help", no_argument, 0, 'h'},
      {"input_file", required_argument, 0, 'f'},
      {"max_entries", required_argument, 0, 'e'},
      {"mesh", required_argument, 0, 'm'},
      {"flux", required_argument, 0, 1},
      {"limiter", required_argument, 0, 2},
      {"boundary", required_argument, 0, 3},
      {"precision", required_argument, 0, 4},
      {"order", required_argument, 0, 5},
      {"output_dir", required_argument, 0, 6},
      {0, 0, 0, 0}};
  std::string input_file, mesh_file, out_dir = ".";
  int flux = -1, limiter = -1, boundary = -1, precision = -1, order = -1;
  for (;;) {
    int idx = 0;
    const int c = getopt_long(argc, argv, "hf:e:m:", long_options, &idx);
    if (c == -1) break;
    switch (c) {
      case 'h': usage(argv[0]); return 0;
      case 'f': input_file = optarg; break;
      case 'e': break;
      case 'm': mesh_file = optarg; break;
      case 1:
        flux = !std::strcmp(optarg, "hlle") ? FVH_FLUX_HLLE
               : !std::strcmp(optarg, "rusanov") ? FVH_FLUX_RUSANOV
               : !std::strcmp(optarg, "hllc") ? FVH_FLUX_HLLC : -2;
        break;
      case 2:
        limiter = !std::strcmp(optarg, "barth_jespersen") ? FVH_LIMITER_BARTH_JESPERSEN
                  : !std::strcmp(optarg, "none") ? FVH_LIMITER_NONE : -2;
        break;
      case 3:
        boundary = !std::strcmp(optarg, "wall") ? FVH_BOUNDARY_WALL
                   : !std::strcmp(optarg, "outflow") ? FVH_BOUNDARY_OUTFLOW : -2;
        break;
      case 4:
        precision = !std::strcmp(optarg, "fp64") ? FVH_PRECISION_FP64
                    : !std::strcmp(optarg, "mixed") ? FVH_PRECISION_MIXED : -2;
        break;
      case 5: order = std::atoi(optarg); break;
      case 6: out_dir = optarg; break;
      default: usage(argv[0]); return 2;
    }
  }
  if (flux == -2 || limiter == -2 || boundary == -2 || precision == -2 ||
      (order != -1 && order != 1 && order != 2)) {
    usage(argv[0]);
    return 2;
  }

  // input file (driver.h:185-196)
  fvh_input *in = nullptr;
  if (!input_file.empty()) {
    std::printf("Using input file \"%s\".\n", input_file.c_str());
    char err[512] = {0};
    const fvh_status st = fvh_input_load(input_file.c_str(), err, sizeof(err), &in);
    if (st != FVH_OK) {
      std::fprintf(stderr, "flecsale_hydro: %s\n", err[0] ? err : fvh_status_string(st));
      return 1;
    }
  }

  // mesh: --mesh, else the input's mesh table
  fvh_host_mesh *hm = nullptr;
  fvh_status st;
  if (!mesh_file.empty())
    st = fvh_host_mesh_read_exodus(mesh_file.c_str(), &hm);
  else if (in)
    st = fvh_input_mesh(in, &hm);
  else
    st = FVH_ERR_INVALID_ARGUMENT;
  if (st != FVH_OK) {
    fvh_input_destroy(in);
    return fail(mesh_file.empty() ? "no mesh (pass --mesh or a hydro.mesh box table)"
                                  : mesh_file.c_str(),
                st);
  }
  fvh_mesh_view hv;
  fvh_host_mesh_view(hm, &hv);
  const int D = hv.dim, nc = hv.num_cells;

  // parameters: the compile-time defaults of {2d,3d}/inputs.cc, then the input
  fvh_params p;
  fvh_params_default(&p, D);
  int64_t max_steps = D == 2 ? 20 : 12;
  char prefix[256];
  std::snprintf(prefix, sizeof(prefix), "%s", D == 2 ? "shock_box_2d" : "shock_box_3d");
  if (in) {
    st = fvh_input_params(in, &p, &max_steps, nullptr);
    if (st != FVH_OK) return fail("input parameters", st);
    fvh_input_string(in, "hydro.prefix", prefix, sizeof(prefix));
  }
  if (flux >= 0) p.flux_kind = flux;
  if (limiter >= 0) p.limiter = limiter;
  if (boundary >= 0) p.boundary = boundary;
  if (precision >= 0) p.precision = precision;
  if (order > 0) p.order = order;

  // initial conditions: hydro.ics, else the shock box of inputs.cc
  std::vector<double> planes((size_t)(5 + D) * nc);
  st = in ? fvh_input_initial_state(in, hm, &p, 0.0, planes.data())
          : fvh_host_initial_state(FVH_PROBLEM_SHOCK_BOX, hm, &p, 0, planes.data());
  if (st != FVH_OK) return fail("initial conditions", st);

  // device: mesh, state, solver; the time loop of driver.h:317-413
  fvh_device_mesh *dm = nullptr;
  fvh_device_state *ds = nullptr;
  fvh_solver *s = nullptr;
  if ((st = fvh_device_mesh_create(hm, &dm)) != FVH_OK) return fail("device mesh", st);
  if ((st = fvh_device_state_create(D, nc, &ds)) != FVH_OK) return fail("device state", st);
  const fvh_state_view *sv = fvh_device_state_view(ds);
  if ((st = fvh_state_upload(sv, D, nc, planes.data(), nullptr)) != FVH_OK)
    return fail("upload", st);
  if ((st = fvh_solver_create(fvh_device_mesh_view(dm), &p, &s)) != FVH_OK)
    return fail("solver", st);
  const fvh_stream_t fs = nullptr;  // the legacy default stream
  const auto t0 = std::chrono::steady_clock::now();
  int64_t done = 0;
  st = fvh_solver_run(s, sv, max_steps, 0, (int32_t)(max_steps > 0 ? max_steps : 1), &done, fs);
  double soln_time = 0;
  int64_t bad = -1;
  const fvh_status chk = fvh_solver_check(s, fs, &soln_time, &bad);
  const double wall =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (st != FVH_OK || chk != FVH_OK) {
    std::fprintf(stderr, "flecsale_hydro: %s (cell %lld)\n",
                 fvh_status_string(st != FVH_OK ? st : chk), (long long)bad);
    return 1;
  }
  std::printf("Final solution time is %.2e after %lld steps.\n", soln_time, (long long)done);
  std::printf("Elapsed wall time is %.4fs.\n", wall);

  // regression dump (driver.h:441-445)
  if ((st = fvh_state_download(sv, D, nc, planes.data(), fs)) != FVH_OK)
    return fail("download", st);
  fvh_solver_check(s, fs, nullptr, nullptr);  // synchronises the stream
  const std::string path = out_dir + "/" + prefix + "-solution_rank000000.txt";
  if ((st = fvh_dump_write(path.c_str(), hm, planes.data(), soln_time, done)) != FVH_OK)
    return fail(path.c_str(), st);

  fvh_solver_destroy(s);
  fvh_device_state_destroy(ds);
  fvh_device_mesh_destroy(dm);
  fvh_host_mesh_destroy(hm);
  fvh_input_destroy(in);
  return 0;
}
