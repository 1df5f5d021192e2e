// Mixed-precision form of the hydro step: FP32 reconstruction and Riemann
// fluxes; FP64 cell state, conservative update and dt reduction.
#pragma once

#include <cuda_runtime.h>

#include "flecsale_gb300.h"

namespace fvh {
namespace mixed {

struct workspace;

fvh_status create(const fvh_mesh_view &m, const fvh_params &p, workspace **out);
void destroy(workspace *w);

// Workspace sized for up to (cells, faces, vertices); setup_geometry derives
// its FP32 geometry from a mesh within those bounds (stream-ordered).
fvh_status create_capacity(int dim, int64_t cells, int64_t faces, int64_t vertices,
                           workspace **out);
cudaError_t setup_geometry(workspace *w, const fvh_mesh_view &m, cudaStream_t st);

// Called after each kernel launch of a step when profiling (name is static).
struct launch_mark {
  void (*fn)(void *ctx, const char *name) = nullptr;
  void *ctx = nullptr;
  void operator()(const char *name) const {
    if (fn) fn(ctx, name);
  }
};

// Launch shape of the cell kernels (picked by the autotuner).  Schedules 0
// and 1 and every block size / cells per thread give the same results bit for
// bit; schedule 2 sums each cell's face fluxes in another order.
struct launch_shape {
  int block = 128;          // threads per block: 128 or 256
  int cells_per_thread = 1; // grid = ceil(cells / (block * cells_per_thread)), grid-stride
  bool staged = false;      // 2D single mesh: gradients from records staged in shared
                            // memory by the bulk-copy engine (gradients_staged_kernel);
                            // the same bits as the global-memory gather
  int schedule = 0;         // 0: cell-centric (each cell evaluates its faces' fluxes);
                            // 1: one flux per face into an array, then a cell gather;
                            // 2: face colouring (single mesh only): per colour, one
                            //    flux per face added to its cells' sums, then the update
};

// Candidate shapes the autotuners time (the batch form skips schedule 2).
constexpr int kNumShapes = 9;
constexpr launch_shape kShapes[kNumShapes] = {
    {128, 1, false, 0}, {256, 1, false, 0}, {128, 2, false, 0}, {256, 2, false, 0},
    {128, 1, false, 1}, {256, 1, false, 1}, {128, 2, false, 1}, {128, 1, false, 2},
    {256, 1, false, 2}};
// Interleaved timing rounds per shape in the autotuners (each shape keeps its
// fastest round).
constexpr int kAutotuneRounds = 2;

// Number of face colours of a workspace made by create() (0 for the batch's).
int colours(const workspace *w);
// Whether the staged gradients serve this workspace's mesh (2D single mesh
// whose chunks fit the shared-memory stages).
bool staging(const workspace *w);

// Steps of one run on a state nothing else writes in between: the corrector
// of a step can also write the next step's FP32 pack and dt (the same bits
// pack_dt computes from the new FP64 state), and the next step then skips
// pack_dt.  A step with pack_first = false must follow one with write_next.
//
// src / out (optional, host-mapped views for callers holding the state in host
// memory): pack_dt reads the state from src and stores it into the device
// state as it packs it; the corrector also writes the new state to out.
struct step_flags {
  bool pack_first = true;   // run pack_dt (the pack and dt from the FP64 state)
  bool write_next = false;  // the corrector writes the next step's pack and dt
  const fvh_state_view *src = nullptr;
  const fvh_state_view *out = nullptr;
};

// One full time step (dt + two half-dt stages) on the FP64 state.
cudaError_t step(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                 const fvh_state_view &s, double *soln_time, double *dt,
                 double *partial, int dt_blocks, fvh_device_status *status,
                 cudaStream_t st, const launch_mark &mark = launch_mark(),
                 const launch_shape &shape = launch_shape(), step_flags f = step_flags());

// Kernel launches per step.
int launches_per_step(const fvh_params &p);
int launches_per_step(const fvh_params &p, const launch_shape &sh, step_flags f = step_flags(),
                      int ncolours = 0);
int launches_per_step_batch(const fvh_params &p, const launch_shape &sh, step_flags f = step_flags());

// Independent problems concatenated into one mesh: problem k owns the cells
// [first_cell[k], first_cell[k+1]).  All arrays are device memory.
struct problem_map {
  const int *cell_problem = nullptr;   // [cells]; null: one problem
  const int *first_cell = nullptr;     // [P+1]
  int nproblems = 1;
  const double *cfl = nullptr;         // [P]
  const double *final_time = nullptr;  // [P]
  double *t = nullptr;                 // [P] solution time
  double *dt = nullptr;                // [P]
  unsigned *dtinv_bits = nullptr;      // [P] max (a+|v.n|)A/V as FP32 bits; reset each step
  fvh_device_status *status = nullptr; // [P]
};

// One time step of every problem of the batch (per-problem dt and time).
// With f.write_next the corrector writes the next step's pack and per-problem
// CFL maxima; a step with f.pack_first = false must follow such a step.
cudaError_t step_batch(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                       const fvh_state_view &s, const problem_map &pm,
                       const launch_shape &shape, cudaStream_t st,
                       const launch_mark &mark = launch_mark(), step_flags f = step_flags());

// Diagnostic: hi/lo of the integer-pipe FP64 -> double-float split, the FP64
// -> FP32 conversion and the FP32 -> FP64 conversion of hi, for x[0..n).
cudaError_t debug_split(const double *x, int64_t n, float *hi, float *lo, float *h2,
                        double *back, cudaStream_t st);

}  // namespace mixed
}  // namespace fvh
