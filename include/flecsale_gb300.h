/*
 * flecsale_gb300 — C ABI of the GB300 (sm_103a) Eulerian finite-volume hydro step.
 *
 * This header is the drop-in boundary for the hydro index tasks of FleCSALE's
 * Eulerian solver (apps/hydro).  Each task entry point below replaces one FleCSI
 * leaf task registered at apps/hydro/tasks.h:857-868 and launched from the time
 * loop in apps/hydro/driver.h:317-413.  The reference passes FleCSI field
 * accessors; this ABI passes plain structs of device pointers (one SoA plane per
 * field component, the reference's "one array per field" registration of
 * apps/hydro/driver.h:33-158) plus counts.  Nothing here uses C++ or CUDA types.
 *
 * Conventions
 *  - All arrays named in fvh_mesh_view / fvh_state_view / fvh_gradient_view /
 *    fvh_flux_view are caller-owned device memory (the fvh_device_* helpers can
 *    allocate them).  Step calls never allocate.
 *  - Every call is asynchronous and stream-ordered on the given stream; no call in
 *    the time loop synchronises with the host.  Errors found by a kernel (the
 *    reference's THROW_RUNTIME_ERROR at tasks.h:366-367 and tasks.h:654-655) are
 *    recorded in a device status word (fvh_device_status) and read by the host
 *    whenever it chooses; launch/argument errors are returned as fvh_status.
 *  - Results are deterministic: no floating-point atomics are used anywhere; the
 *    face-to-cell accumulation is a cell-centric gather in the cell's face order.
 *  - dim is 2 or 3.  Index arrays are int32.
 *  - Threads: a handle (fvh_solver, fvh_batch, fvh_input, meshes and states)
 *    is used by one thread at a time, since a solver or batch keeps per-stream
 *    CUDA graphs and pinned scalars; distinct handles may be used concurrently
 *    from different threads on different streams.  The task entry points keep
 *    no state between calls (fvh_evaluate_time_step_noalloc excepted: its
 *    calls share one scratch array, see there).
 */
#ifndef FLECSALE_GB300_H
#define FLECSALE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FVH_ABI_VERSION 1

/* A cudaStream_t; 0 is the legacy default stream. */
typedef struct CUstream_st *fvh_stream_t;

/* ------------------------------------------------------------------------- */
/* Status codes                                                               */
/* ------------------------------------------------------------------------- */
typedef enum fvh_status {
  FVH_OK = 0,
  FVH_ERR_INVALID_ARGUMENT = 1,   /* null pointer, bad dim/kind, size mismatch   */
  FVH_ERR_CUDA = 2,               /* a CUDA runtime call failed                  */
  FVH_ERR_INFINITE_DT = 3,        /* tasks.h:366-367 "infinite delta t"          */
  FVH_ERR_NEGATIVE_STATE = 4,     /* tasks.h:654-655 negative density or energy  */
  FVH_ERR_UNSUPPORTED = 5,        /* mesh cell shape / option not supported      */
  FVH_ERR_NO_DEVICE = 6,          /* no CUDA device visible                       */
  FVH_ERR_OUT_OF_MEMORY = 7,      /* a device or host allocation failed; no C++
                                     exception ever crosses this ABI            */
  FVH_ERR_CAPACITY = 8,           /* a request exceeds a fixed capacity           */
  FVH_ERR_TIMEOUT = 9             /* a kernel's bounded wait on its own data
                                     copies ran out (the kernel stopped early)   */
} fvh_status;

/* Human-readable text for an fvh_status value (static storage). */
const char *fvh_status_string(int32_t status);

/* ABI version of the loaded library (FVH_ABI_VERSION when built). */
int32_t fvh_abi_version(void);

/* ------------------------------------------------------------------------- */
/* Physics / scheme parameters                                                */
/* ------------------------------------------------------------------------- */
typedef enum fvh_flux_kind {
  FVH_FLUX_HLLE = 0,     /* reference default: flux_function -> hlle_flux,
                            apps/hydro/types.h:118-125, flecsale/eqns/flux.h:79-106 */
  FVH_FLUX_RUSANOV = 1,  /* flecsale/eqns/flux.h:51-65                               */
  FVH_FLUX_HLLC = 2      /* not in the reference: Toro's HLLC with the HLLE
                            wave-speed estimates (flux.h:82-86)                      */
} fvh_flux_kind;

typedef enum fvh_limiter_kind {
  FVH_LIMITER_BARTH_JESPERSEN = 0, /* reference vertex limiter, tasks.h:267-299 */
  FVH_LIMITER_NONE = 1             /* unlimited least-squares gradients         */
} fvh_limiter_kind;

typedef enum fvh_boundary_kind {
  FVH_BOUNDARY_WALL = 0,   /* reference: boundary_flux -> wall_flux,
                              apps/hydro/types.h:132-137, euler_eqns.h:313-324 */
  FVH_BOUNDARY_OUTFLOW = 1 /* not in the reference: transmissive boundary, the
                              face flux is the physical flux of the reconstructed
                              interior state, euler_eqns.h:274-304            */
} fvh_boundary_kind;

typedef enum fvh_precision {
  FVH_PRECISION_FP64 = 0,  /* everything in FP64 (reference arithmetic order)      */
  FVH_PRECISION_MIXED = 1  /* FP32 reconstruction + Riemann flux, FP64 state,
                              update, totals and dt                                */
} fvh_precision;

typedef struct fvh_params {
  int32_t dim;            /* 2 or 3                                               */
  int32_t flux_kind;      /* fvh_flux_kind (interior faces); walls use wall_flux  */
  int32_t limiter;        /* fvh_limiter_kind                                     */
  int32_t order;          /* 2 = MUSCL (reference); 1 = first order (zero grads)  */
  int32_t recon_swap_ep;  /* 1 = reproduce the reference's reconstruction, which
                             adds grad(e) to the face pressure and grad(p) to the
                             face energy (tasks.h:429-430, 448-449); 0 = textbook */
  int32_t precision;      /* fvh_precision                                        */
  int32_t boundary;       /* fvh_boundary_kind for faces with one cell            */
  int32_t reserved;       /* must be 0                                            */
  double gamma;           /* ideal gas ratio of specific heats (ideal_gas.h:42)   */
  double cv;              /* specific heat at constant volume                      */
  double cfl;             /* CFL number (inputs.h:64)                              */
  double final_time;      /* dt is clamped to final_time - t (tasks.h:343,373)    */
} fvh_params;

/* Fill p with the reference's 2D shock-box defaults (apps/hydro/2d/inputs.cc:27-42):
 * HLLE, Barth-Jespersen, 2nd order, swap on, FP64, walls, gamma 1.4, cv 1,
 * CFL 0.5 (1/3 in 3D, 3d/inputs.cc:108), t_f 0.2. */
void fvh_params_default(fvh_params *p, int32_t dim);

/* ------------------------------------------------------------------------- */
/* Views of device memory                                                     */
/* ------------------------------------------------------------------------- */

/* Mesh topology + geometry (burton mesh queries, apps/hydro/types.h:33 and the
 * calls made in tasks.h).  Geometry is FP64, one plane per component. */
typedef struct fvh_mesh_view {
  int32_t dim;
  int32_t num_cells;
  int32_t num_faces;
  int32_t num_vertices;
  /* cells(f): face_cells[2f] = cells(f)[0], face_cells[2f+1] = cells(f)[1] or -1
   * for a boundary face.  The face normal points out of cells(f)[0]. */
  const int32_t *face_cells;
  /* faces(c) in the reference's iteration order, CSR.  Each entry is f when
   * c == cells(f)[0] (flux subtracted) and ~f (= -f-1) otherwise (flux added). */
  const int32_t *cell_face_offsets;   /* [num_cells+1] */
  const int32_t *cell_faces;
  /* cell_vertex_neighbors(c) (tasks.h:190), CSR in the reference's order. */
  const int32_t *cell_nbr_offsets;    /* [num_cells+1] */
  const int32_t *cell_nbrs;
  /* vertices(c) (tasks.h:270), CSR. */
  const int32_t *cell_vertex_offsets; /* [num_cells+1] */
  const int32_t *cell_vertices;
  const double *cell_centroid[3];     /* c->centroid()   */
  const double *cell_volume;          /* c->volume()     */
  const double *face_centroid[3];     /* f->centroid()   */
  const double *face_normal[3];       /* f->normal(), unit, out of cells(f)[0] */
  const double *face_area;            /* f->area()       */
  const double *vertex_coord[3];      /* v->coordinates() */
} fvh_mesh_view;

/* Cell state: the six hydro fields of driver.h:215-224 (d, v, e, p, T, a). */
typedef struct fvh_state_view {
  double *density;
  double *velocity[3];
  double *internal_energy;
  double *pressure;
  double *temperature;
  double *sound_speed;
} fvh_state_view;

/* Limited cell gradients (driver.h:228-232); g[k] is d/dx_k.
 * velocity[d][k] = d v_d / d x_k, the reference's grad_v(c)[d][k]. */
typedef struct fvh_gradient_view {
  double *density[3];
  double *velocity[3][3];
  double *internal_energy[3];
  double *pressure[3];
  double *sound_speed[3];
} fvh_gradient_view;

/* Area-scaled face fluxes (flux_data_t, driver.h:226): mass, momentum[dim], energy. */
typedef struct fvh_flux_view {
  double *mass;
  double *momentum[3];
  double *energy;
} fvh_flux_view;

/* Device status word.  Kernels record the first offending cell with an integer
 * atomicMin on key = (cell << 8) | code, so the result does not depend on thread
 * order.  FVH_STATUS_CLEAR means "no error".  Decode with fvh_status_decode. */
typedef unsigned long long fvh_device_status;
#define FVH_STATUS_CLEAR (~0ull)
void fvh_status_decode(fvh_device_status s, int32_t *code, int64_t *cell);

/* ------------------------------------------------------------------------- */
/* Task entry points (stream-ordered, asynchronous, no allocation)            */
/* ------------------------------------------------------------------------- */

/* Bytes of device workspace fvh_evaluate_time_step needs for num_cells cells. */
size_t fvh_time_step_workspace_bytes(int32_t num_cells);

/* Replaces evaluate_time_step (tasks.h:331-376) plus the min-reduction over
 * colours (driver.h:329-332): d_dt[0] = min(CFL / max_{c,f in c}
 * (a_c + |v_c.n_f|) A_f / V_c, final_time - d_soln_time[0]).  A non-positive
 * maximum records FVH_ERR_INFINITE_DT in d_status.  d_workspace must hold
 * fvh_time_step_workspace_bytes(num_cells) bytes. */
fvh_status fvh_evaluate_time_step(const fvh_mesh_view *mesh,
                                  const fvh_state_view *state,
                                  const fvh_params *params,
                                  const double *d_soln_time, double *d_dt,
                                  void *d_workspace, size_t workspace_bytes,
                                  fvh_device_status *d_status,
                                  fvh_stream_t stream);

/* No counterpart in the reference.  Same result as fvh_evaluate_time_step, for
 * callers that cannot allocate device memory (a task runtime that owns all
 * device memory and hands a task only its field buffers, or a hot loop that
 * must not pay cudaMalloc's implicit synchronisation).  It takes no workspace:
 * the partial maxima live in a 64 KiB array inside the library, which every
 * GPU that loads the library holds until exit.  Meshes with more than
 * fvh_time_step_noalloc_max_cells() = 2,097,152 cells are rejected with
 * FVH_ERR_CAPACITY.  The first call on a device looks up that array's device
 * address (make it before any stream capture).  All calls share the array:
 * calls whose kernels overlap on the GPU (e.g. on two streams) race.  It calls
 * no cudaMalloc, cudaFree or allocating routine. */
fvh_status fvh_evaluate_time_step_noalloc(const fvh_mesh_view *mesh,
                                          const fvh_state_view *state,
                                          const fvh_params *params,
                                          const double *d_soln_time, double *d_dt,
                                          fvh_device_status *d_status,
                                          fvh_stream_t stream);
int32_t fvh_time_step_noalloc_max_cells(void);

/* Replaces evaluate_gradients (tasks.h:145-321): vertex-neighbour least squares
 * gradients of (d, v, e, p, a) with the Barth-Jespersen vertex limiter. */
fvh_status fvh_evaluate_gradients(const fvh_mesh_view *mesh,
                                  const fvh_state_view *state,
                                  const fvh_gradient_view *grads,
                                  const fvh_params *params,
                                  fvh_stream_t stream);

/* Replaces evaluate_fluxes (tasks.h:385-536): per face, reconstruct both sides at
 * the face centroid, Riemann flux (interior) or wall flux (boundary), times area. */
fvh_status fvh_evaluate_fluxes(const fvh_mesh_view *mesh,
                               const fvh_state_view *state,
                               const fvh_gradient_view *grads,
                               const fvh_flux_view *flux,
                               const fvh_params *params, fvh_stream_t stream);

/* Replaces apply_update (tasks.h:589-659) and update_soln_time (tasks.h:545-576):
 * delta_t = d_dt[0]*factor; d_soln_time[0] += delta_t; per cell
 * du = sum over faces(c) of -/+ F_f, du *= delta_t / V_c, conservative update
 * (euler_eqns.h:383-410) and EOS closure (euler_eqns.h:359-375).  A negative
 * density or internal energy records FVH_ERR_NEGATIVE_STATE in d_status. */
fvh_status fvh_apply_update(const fvh_mesh_view *mesh, const fvh_params *params,
                            const double *d_dt, double factor,
                            const fvh_flux_view *flux,
                            const fvh_state_view *state, double *d_soln_time,
                            fvh_device_status *d_status, fvh_stream_t stream);

/* ------------------------------------------------------------------------- */
/* Solver object: one mesh + its work buffers, the whole time step            */
/* ------------------------------------------------------------------------- */
typedef struct fvh_solver fvh_solver;

/* Allocates gradients, fluxes, the dt workspace and the device scalars
 * (solution time, dt, status) for a mesh already in device memory.  The mesh
 * view is copied; the arrays it points to must outlive the solver. */
fvh_status fvh_solver_create(const fvh_mesh_view *mesh, const fvh_params *params,
                             fvh_solver **out);
void fvh_solver_destroy(fvh_solver *s);

/* One full time step of driver.h:325-375 on the state: dt reduction, then the
 * predictor and the corrector (gradients -> fluxes -> update, factor 0.5 each). */
fvh_status fvh_solver_step(fvh_solver *s, const fvh_state_view *state,
                           fvh_stream_t stream);

/* nsteps steps, stream-ordered.  With stop_at_final_time != 0 the host checks the
 * solution time every check_every steps and stops once it reaches final_time
 * (the dt clamp of tasks.h:373 makes the last step land on it).  Within a run
 * (between host checks) the state must not be written by anyone else: in the
 * mixed form a step's corrector prepares the next step's FP32 pack and dt.
 * Results are bitwise those of the same number of fvh_solver_step calls. */
fvh_status fvh_solver_run(fvh_solver *s, const fvh_state_view *state,
                          int64_t nsteps, int32_t stop_at_final_time,
                          int32_t check_every, int64_t *steps_done,
                          fvh_stream_t stream);

/* Device scalars owned by the solver. */
double *fvh_solver_soln_time(fvh_solver *s);
double *fvh_solver_dt(fvh_solver *s);
fvh_device_status *fvh_solver_status(fvh_solver *s);
const fvh_gradient_view *fvh_solver_gradients(fvh_solver *s);
const fvh_flux_view *fvh_solver_fluxes(fvh_solver *s);

/* Kernel launches one fvh_solver_step makes (the CUDA graph's node count). */
int32_t fvh_solver_launches_per_step(const fvh_solver *s);

/* Launch shape of the mixed form's cell kernels: block 128 or 256, cells per
 * thread 1..8, schedule 0 (each cell evaluates its faces' fluxes), 1 (one
 * flux per face into an array, then a cell gather) or 2 (face colouring: for
 * each colour of a greedy colouring in which no two faces of a colour share a
 * cell, one flux per face added to its cells' compensated sums; then the
 * update).  Schedules 0 and 1 and all block sizes / cells per thread give the
 * same bits; schedule 2 adds each cell's fluxes in colour order, so its sums
 * round differently (deterministically).  schedule | FVH_SCHEDULE_STAGED (2D
 * meshes whose cell chunks fit the stages; FVH_ERR_INVALID_ARGUMENT otherwise)
 * takes the gradients from neighbour records staged in shared memory by the
 * bulk-copy engine, with the same bits.  The FP64 form ignores it.  No
 * reference counterpart: the reference's tasks have no launch configuration. */
#define FVH_SCHEDULE_STAGED 4
fvh_status fvh_solver_set_shape(fvh_solver *s, int32_t block, int32_t cells_per_thread,
                                int32_t schedule);

/* Diagnostic of the mixed form's integer-pipe conversions on device arrays of
 * n elements: hi/lo = the double-float split of x (hi + lo = x to about 2^-48),
 * rn32 = x rounded to FP32 (FP32 subnormals flush to zero), hi_as_double = hi
 * converted back to FP64.  No reference counterpart. */
fvh_status fvh_debug_split(const double *x, int64_t n, float *hi, float *lo, float *rn32,
                           double *hi_as_double, fvh_stream_t stream);

/* Diagnostic of the FP64 kernels' integer-pipe arithmetic on device arrays of
 * n elements: out[i] = a[i] op b[i], op 0 = multiply, 1 = add, 2 = subtract,
 * 3 = divide, each correctly rounded to nearest-even on the integer/FP32
 * pipes; op 4..7 = the same four with the FP64 instructions; op 8 / 9 = the
 * FP64 kernels' branch-free multiply / divide, redone with the FP64
 * instruction where they flag an operand; op 10 = the kernels' halving of
 * a[i] (0.5 * a and a / 2; b unused), redone likewise.  All must agree bit
 * for bit with the FP64 instructions on every input.  No reference
 * counterpart. */
fvh_status fvh_debug_sf64(int32_t op, const double *a, const double *b, int64_t n,
                          double *out, fvh_stream_t stream);

/* Times each candidate launch shape (with and without FVH_SCHEDULE_STAGED
 * where the mesh allows it) for trial_steps steps on a scratch copy of
 * `state`, in two interleaved rounds (a shape's figure is its faster
 * round), and keeps the fastest; the state, solution time and status word are
 * left unchanged.  Synchronises; allocates the scratch copy.  No reference
 * counterpart. */
fvh_status fvh_solver_autotune(fvh_solver *s, const fvh_state_view *state, int32_t trial_steps,
                               int32_t *block, int32_t *cells_per_thread, int32_t *schedule,
                               double *best_ms_per_step, fvh_stream_t stream);

/* Kernel launches of fvh_solver_run(s, state, nsteps, 0, ...): in the mixed
 * form the first step computes the FP32 pack and dt from the FP64 state and
 * every later step gets them from the previous step's corrector. */
int64_t fvh_solver_launches_per_run(const fvh_solver *s, int64_t nsteps);

/* Profiling run: nsteps steps, launched as fvh_solver_run launches them but
 * kernel by kernel, with a CUDA event recorded on the stream after every
 * launch.  For each distinct kernel name (at most max_kernels) returns its
 * static name, its mean duration in milliseconds per launch and its number of
 * launches in the nsteps steps.  Synchronises. */
fvh_status fvh_solver_profile(fvh_solver *s, const fvh_state_view *state,
                              int32_t nsteps, int32_t max_kernels,
                              const char **names, double *mean_ms,
                              int32_t *launches, int32_t *nkernels,
                              fvh_stream_t stream);

/* Synchronises the stream, reads the status word and the solution time. */
fvh_status fvh_solver_check(fvh_solver *s, fvh_stream_t stream,
                            double *soln_time, int64_t *bad_cell);

/* Reset the solution time to t and clear the status word (stream-ordered). */
fvh_status fvh_solver_reset(fvh_solver *s, double t, fvh_stream_t stream);

/* ------------------------------------------------------------------------- */
/* Host mesh construction (the burton topology + geometry queries)            */
/* ------------------------------------------------------------------------- */
typedef struct fvh_host_mesh fvh_host_mesh;

/* Build topology and geometry from cell -> vertex lists.
 *  dim 2: each cell is a polygon with vertices listed counter-clockwise.
 *  dim 3: each cell is a hexahedron (8 vertices, Exodus HEX8 order) or a
 *         tetrahedron (4 vertices, Exodus TETRA4 order).
 * vertex_coords is interleaved [num_vertices*dim]. */
fvh_status fvh_host_mesh_create(int32_t dim, int32_t num_vertices,
                                const double *vertex_coords, int32_t num_cells,
                                const int32_t *cell_vertex_offsets,
                                const int32_t *cell_vertices,
                                fvh_host_mesh **out);

/* No reference counterpart (the reference reads its meshes from Exodus files):
 * structured-origin box mesh stored unstructured: n[0] x n[1] (x n[2]) cells on
 * [lo, hi], vertex and cell ids lexicographic with x fastest.  Interior vertices
 * are moved by independent uniform offsets in [-jitter*h_k, +jitter*h_k] per axis
 * (SplitMix64 stream keyed by seed and vertex id); boundary vertices stay put. */
fvh_status fvh_host_mesh_box(int32_t dim, const int32_t *n, const double *lo,
                             const double *hi, double jitter, uint64_t seed,
                             fvh_host_mesh **out);

void fvh_host_mesh_destroy(fvh_host_mesh *m);

/* Read an Exodus II mesh file in the netCDF classic (CDF-1) or 64-bit-offset
 * (CDF-2) encoding: all element blocks connect1..N (QUAD4/SHELL4 as 2D
 * polygons, HEX8, TETRA4), coordinates coordx/coordy[/coordz] or coord.
 * Cell and vertex ids follow the file.  netCDF-4/HDF5 files give
 * FVH_ERR_UNSUPPORTED.  Replaces the flecsi-sp Exodus reader behind the
 * reference's "-m mesh" argument (apps/common/arguments.h:44-52). */
fvh_status fvh_host_mesh_read_exodus(const char *path, fvh_host_mesh **out);

/* Write the regression dump of apps/hydro/tasks.h:771-849 (precision 14,
 * scientific; cells then vertices) for host state planes
 * (d, v[0..dim), e, p, T, a). */
fvh_status fvh_dump_write(const char *path, const fvh_host_mesh *m,
                          const double *host_planes, double soln_time,
                          int64_t iterations);

/* Read a regression dump (the format above and of tasks.h:771-849) back into
 * host state planes (d, v[0..dim), e, p, T, a) of num_cells cells, by local_id:
 * density, internal energy, pressure and velocity as printed (15 significant
 * digits), T = e / cv and a = sqrt(gamma (gamma - 1) e) as
 * update_state_from_energy closes them (euler_eqns.h:359-375).  The header's
 * solution time and iteration count go to *soln_time and *iterations (either
 * may be null).  A dump whose cell count differs, or that is malformed, gives
 * FVH_ERR_INVALID_ARGUMENT.  No reference counterpart (the reference only
 * writes dumps); it lets a run resume from one. */
fvh_status fvh_dump_read(const char *path, int32_t dim, int32_t num_cells, double gamma,
                         double cv, double *host_planes, double *soln_time,
                         int64_t *iterations);

/* EOS closure of caller-provided density, velocity planes [dim][n] and
 * pressure (update_state_from_pressure, euler_eqns.h:333-350) into state
 * planes d, v..., e, p, T, a: the second half of initial_conditions
 * (apps/hydro/tasks.h:58-66). */
fvh_status fvh_host_state_from_dvp(int32_t dim, int32_t n, double gamma, double cv,
                                   const double *density, const double *velocity,
                                   const double *pressure, double *host_planes);

/* No reference counterpart (used by the batched form).  Concatenate meshes of
 * one dimension into one block-diagonal mesh: cells,
 * faces and vertices of mesh k follow those of meshes 0..k-1, with all indices
 * shifted; no connectivity is added between meshes. */
fvh_status fvh_host_mesh_concat(int32_t n, const fvh_host_mesh *const *meshes,
                                fvh_host_mesh **out);

/* Host-memory view of the mesh arrays (valid while m lives). */
fvh_status fvh_host_mesh_view(const fvh_host_mesh *m, fvh_mesh_view *out);

/* Lengths of the CSR index arrays. */
fvh_status fvh_host_mesh_nnz(const fvh_host_mesh *m, int64_t *cell_faces,
                             int64_t *cell_nbrs, int64_t *cell_vertices);

/* ------------------------------------------------------------------------- */
/* Initial conditions (setup)                                                 */
/* ------------------------------------------------------------------------- */
typedef enum fvh_problem_kind {
  FVH_PROBLEM_SHOCK_BOX = 0,   /* (0.125, 0, 0.1) where every x_k < 0, else (1, 0, 1):
                                  apps/hydro/2d/inputs.cc:45-60, 3d/inputs.cc:120-137 */
  FVH_PROBLEM_SOD = 1,         /* x < 0.5: (1, 0, 1); else (0.125, 0, 0.1)             */
  FVH_PROBLEM_FOUR_QUADRANT = 2, /* 2D quadrants about (0.5, 0.5), (d, u, v, p):
                                  NE (1.5,0,0,1.5) NW (0.5323,1.206,0,0.3)
                                  SW (0.138,1.206,1.206,0.029) SE (0.5323,0,1.206,0.3) */
  FVH_PROBLEM_INNER_CUBE = 3,  /* every x_k < 0.5: (1, 0, 1); else (0.125, 0, 0.1)     */
  FVH_PROBLEM_KELVIN_HELMHOLTZ = 4, /* d = 2 (|y-0.5| < 0.25) else 1, u = +0.5 / -0.5,
                                  v = 0.01 sin(4 pi x) + 1e-3 U[-1,1) (seeded), p = 2.5 */
  FVH_PROBLEM_UNIFORM = 5      /* (1, 0, 1) everywhere                                  */
} fvh_problem_kind;

/* Per-cell (d, v, p) of the problem at the cell centroid, closed with the ideal
 * gas (update_state_from_pressure, euler_eqns.h:333-350).  host_planes receives
 * 5+dim planes of num_cells doubles: d, v[0..dim), e, p, T, a. */
fvh_status fvh_host_initial_state(int32_t kind, const fvh_host_mesh *m,
                                  const fvh_params *p, uint64_t seed,
                                  double *host_planes);

/* ------------------------------------------------------------------------- */
/* Device memory helpers (setup only, never called inside a step)             */
/* ------------------------------------------------------------------------- */
/* In the reference the FleCSI data model owns all field storage (fields
 * registered at apps/hydro/driver.h:33-158); these helpers are the optional
 * owner for callers that do not manage device memory themselves. */
typedef struct fvh_device_mesh fvh_device_mesh;

/* Copy a host mesh to device memory. */
fvh_status fvh_device_mesh_create(const fvh_host_mesh *m, fvh_device_mesh **out);
void fvh_device_mesh_destroy(fvh_device_mesh *dm);
const fvh_mesh_view *fvh_device_mesh_view(const fvh_device_mesh *dm);

/* State planes for num_cells cells in one device allocation. */
typedef struct fvh_device_state fvh_device_state;
fvh_status fvh_device_state_create(int32_t dim, int32_t num_cells,
                                   fvh_device_state **out);
void fvh_device_state_destroy(fvh_device_state *ds);
const fvh_state_view *fvh_device_state_view(const fvh_device_state *ds);

/* Host <-> device copies of a whole state.  Host layout: 5+dim planes of
 * num_cells doubles in the order d, v[0..dim), e, p, T, a. */
fvh_status fvh_state_upload(const fvh_state_view *dst, int32_t dim,
                            int32_t num_cells, const double *host_planes,
                            fvh_stream_t stream);
fvh_status fvh_state_download(const fvh_state_view *src, int32_t dim,
                              int32_t num_cells, double *host_planes,
                              fvh_stream_t stream);

/* No reference counterpart.  End-to-end call for callers that hold the state
 * in host memory: upload the
 * state, advance nsteps time steps, download it, then synchronise.  Solution
 * time in/out through *soln_time.  With pinned host planes (cudaHostAlloc /
 * cudaHostRegister) the first kernel (the mixed form's pack, the FP64 form's
 * dt) reads the state from host memory and the last update writes the new
 * state to it directly, overlapping the transfers with the step; the
 * temperature plane is not read (the step rewrites it).  The results and the
 * device state afterwards are the same as with copies. */
fvh_status fvh_solver_advance_host(fvh_solver *s, const fvh_state_view *dev_state,
                                   double *host_planes, int64_t nsteps,
                                   double *soln_time, fvh_stream_t stream);


/* ------------------------------------------------------------------------- */
/* Input files: the Lua "hydro" table of apps/hydro/inputs.h:100-135          */
/* ------------------------------------------------------------------------- */
typedef struct fvh_input fvh_input;

/* Parse and run a Lua input file (replaces inputs_t::load, inputs.h:83-97;
 * the subset FleCSALE inputs use: tables, numbers, strings, and functions with
 * locals, if/elseif/else, numeric for, while, multiple returns and the math
 * library).  On failure *out is null and err (when given) holds
 * "file:line: message"; the file must define a table "hydro". */
fvh_status fvh_input_load(const char *path, char *err, size_t err_len, fvh_input **out);
fvh_status fvh_input_load_string(const char *text, char *err, size_t err_len,
                                 fvh_input **out);
void fvh_input_destroy(fvh_input *in);

/* Number or string at a path below the globals, e.g. "hydro.CFL",
 * "hydro.eos.gas_constant", "hydro.mesh.dimensions[2]".  Numeric strings
 * ("1e6", as output_freq in shock_box_2d.lua) read as numbers, as Lua converts
 * them.  FVH_ERR_INVALID_ARGUMENT when absent or of another type. */
fvh_status fvh_input_number(const fvh_input *in, const char *path, double *value);
fvh_status fvh_input_string(const fvh_input *in, const char *path, char *buf, size_t len);

/* The keys inputs.h:112-132 reads: CFL, final_time, eos = {type = "ideal_gas",
 * gas_constant, specific_heat} into p (absent keys keep p's values), and
 * max_steps and output_freq into the counters (either may be null).  Another
 * eos type returns FVH_ERR_UNSUPPORTED (inputs.h:129-131).  The merged
 * parameters are validated, so the values p brings in for keys the file does
 * not set must be valid too: a merged value out of range (a non-positive or
 * non-finite CFL, gamma <= 1, cv <= 0, a NaN final time, a negative or
 * fractional count) returns FVH_ERR_INVALID_ARGUMENT and leaves p and the
 * counters unchanged.  fvh_params_default gives valid values. */
fvh_status fvh_input_params(const fvh_input *in, fvh_params *p, int64_t *max_steps,
                            int64_t *output_freq);

/* hydro.mesh = {type = "box", dimensions = {nx, ny[, nz]}, xmin = {..}, xmax = {..}}
 * (apps/hydro/3d/shock_box_3d.lua) as an unjittered box mesh. */
fvh_status fvh_input_mesh(const fvh_input *in, fvh_host_mesh **out);

/* Evaluate hydro.ics(x, y[, z], t) at every cell centroid; it returns density,
 * {velocity}, pressure, closed with the ideal gas as initial_conditions does
 * (tasks.h:46-68).  host_planes: (5+dim) x num_cells. */
fvh_status fvh_input_initial_state(const fvh_input *in, const fvh_host_mesh *m,
                                   const fvh_params *p, double t, double *host_planes);

/* ------------------------------------------------------------------------- */
/* Batched form: independent meshes advanced together (mixed precision)      */
/* ------------------------------------------------------------------------- */
/* No counterpart in the reference, whose driver advances one mesh per colour.
 * A batch holds up to max_problems meshes with at most the given total cells,
 * faces and vertices, concatenated block-diagonally in device memory; each
 * problem has its own CFL number, final time, solution time, dt and status.
 * One fvh_batch_step advances every problem by nsteps steps in one CUDA-graph
 * launch; a problem at its final time gets dt = 0.  Results of a problem do not
 * depend on the other problems in the batch. */
typedef struct fvh_batch fvh_batch;

/* params: shared scheme (precision must be FVH_PRECISION_MIXED; dim, flux,
 * limiter, order, swap, boundary, gamma, cv). */
fvh_status fvh_batch_create(const fvh_params *params, int64_t max_cells,
                            int64_t max_faces, int64_t max_vertices,
                            int32_t max_problems, fvh_batch **out);
void fvh_batch_destroy(fvh_batch *b);

/* Replace the batch's problems by n meshes.  keep[k] >= 0 carries the device
 * state and solution time of problem keep[k] of the previous assignment (same
 * cell count) into new problem k; keep == NULL or keep[k] < 0 leaves problem k
 * to be set with fvh_batch_set_state.  Synchronises the stream. */
fvh_status fvh_batch_assign(fvh_batch *b, int32_t n, const fvh_host_mesh *const *meshes,
                            const double *cfl, const double *final_time,
                            const int32_t *keep, fvh_stream_t stream);

/* Same as fvh_batch_assign for meshes already in device memory
 * (fvh_device_mesh_create): the concatenation runs on the device, so changing
 * the set of problems costs no host work or host-to-device traffic for the
 * problems that stay. */
fvh_status fvh_batch_assign_device(fvh_batch *b, int32_t n,
                                   const fvh_device_mesh *const *meshes,
                                   const double *cfl, const double *final_time,
                                   const int32_t *keep, fvh_stream_t stream);

/* Host planes (d, v[0..dim), e, p, T, a; one plane per field, problem cells)
 * in and out of problem k; set_state also sets its solution time.  Both
 * synchronise the stream. */
fvh_status fvh_batch_set_state(fvh_batch *b, int32_t k, const double *host_planes,
                               double t, fvh_stream_t stream);
fvh_status fvh_batch_get_state(fvh_batch *b, int32_t k, double *host_planes,
                               fvh_stream_t stream);

/* Advance every problem nsteps steps (one CUDA graph per step count). */
fvh_status fvh_batch_step(fvh_batch *b, int32_t nsteps, fvh_stream_t stream);

/* Synchronise; per problem: solution time, status code and first bad cell
 * (problem-local id).  Returns the first non-OK code, if any. */
fvh_status fvh_batch_query(fvh_batch *b, double *times, int32_t *codes,
                           int64_t *bad_cells, fvh_stream_t stream);

/* Launch shape of the cell kernels: threads per block (128 or 256), cells per
 * thread (1..8) and flux schedule (0: each cell evaluates the fluxes of its
 * faces; 1: one flux per face into an array, then a cell-centric gather).  All
 * shapes give the same results bit for bit. */
fvh_status fvh_batch_set_shape(fvh_batch *b, int32_t block, int32_t cells_per_thread,
                               int32_t schedule);

/* Autotuner: times each launch shape (threads per block x cells per thread x
 * schedule) for trial_steps steps on the current problems, keeps the fastest
 * and restores the state, times and status words, so tuning does not change
 * the results.  The winner is appended to a cache file (FVH_AUTOTUNE_CACHE,
 * default $HOME/.cache/flecsale_gb300_autotune.txt) keyed by device, scheme
 * and size class; with use_cache != 0 a cached entry is applied without
 * measuring (best_ms_per_step is then -1).  Allocates a temporary copy of the
 * state. */
fvh_status fvh_batch_autotune(fvh_batch *b, int32_t trial_steps, int32_t use_cache,
                              int32_t *block, int32_t *cells_per_thread,
                              int32_t *schedule, double *best_ms_per_step,
                              fvh_stream_t stream);

int32_t fvh_batch_num_problems(const fvh_batch *b);
int64_t fvh_batch_num_cells(const fvh_batch *b);
/* Kernel launches of a step after the first of one fvh_batch_step call (the
 * first adds one: it computes the FP32 pack and CFL maxima from the FP64
 * state; later steps get them from the previous step's corrector). */
int32_t fvh_batch_launches_per_step(const fvh_batch *b);

#ifdef __cplusplus
}
#endif
#endif /* FLECSALE_GB300_H */
