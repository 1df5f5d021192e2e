// Plain FP64 kernels of the Eulerian hydro step (sm_103a).
//
// This translation unit is compiled with --fmad=false: every multiply and add
// below rounds separately, in the order the reference writes them, so the
// results are bit-identical to the reference arithmetic of
//   evaluate_time_step  apps/hydro/tasks.h:331-376
//   evaluate_gradients  apps/hydro/tasks.h:145-321
//   evaluate_fluxes     apps/hydro/tasks.h:385-464
//   apply_update        apps/hydro/tasks.h:589-659
// with the physics of flecsale/eqns/euler_eqns.h and flecsale/eqns/flux.h and
// the ideal gas of flecsale/eos/ideal_gas.h (IEEE division and square root are
// correctly rounded on both CPU and GPU).
//
// Layout: every field component is its own FP64 plane (SoA), so a warp's 32
// consecutive cells or faces read 256 contiguous bytes per plane.  Neighbour
// gathers follow the CSR lists in the reference's iteration order; with
// lexicographic numbering the neighbours of a warp's cells share cache lines and
// are served from L1/L2 after the first touch.
//
// Pipes: GB300 issues 2 FP64 operations per clock per SM.  Most products and
// every quotient below are computed on the integer/FP32 pipes by the
// correctly rounded routines of fvh_sf64.cuh, while most sums and differences
// stay on the FP64 pipe; each kernel moves a part of one kind to the other
// pipe so that both are loaded alike (fp64_products, add_call).  Comparisons,
// minima and maxima run on integer order keys.  Both pipes round to
// nearest-even exactly as IEEE binary64 does, so the bits are unchanged, and
// they work at the same time.  Each unit of work (a cell or a
// face) is evaluated optimistically with the branch-free integer forms
// (arith_opt); if any operand was of a kind they do not handle (subnormal,
// infinite, NaN, beyond 2^+-500) the unit is evaluated again with the FP64
// instructions (arith_hw) and that result is kept.
//
// Code size: the integer forms inline to tens of instructions per product, so
// a fully unrolled kernel outgrows the SM's instruction cache and its warps
// stall on instruction fetch.  The kernels keep their neighbour and vertex
// loops rolled, evaluate each physical flux once per side (selecting the
// state instead of branching into copies), and take products, quotients and
// the FP64 redo of a rare unit in out-of-line calls (2.27 -> 1.77 ms per 2D
// step on the 1024^2 workload; the pipe balance and the variable groups of
// the gradients below took it on to 1.49 ms).
#include <cuda_runtime.h>

#include <cstdint>

#include "flecsale_gb300.h"
#include "fvh_kernels.h"
#include "fvh_sf64.cuh"

namespace fvh {
namespace plain {

// Products and quotients in out-of-line calls (a call costs a few
// instructions; inlining them everywhere made the kernels too large for the
// instruction cache).  Each returns its result with the flag that an operand
// was left to the hardware.
struct flagged {
  double q;
  unsigned rare;
};
__device__ __noinline__ flagged mul_call(double a, double b) {
  flagged r;
  r.rare = 0;
  r.q = sf64::mul_opt(a, b, r.rare);
  return r;
}
__device__ __noinline__ flagged div_call(double a, double b) {
  flagged r;
  r.rare = 0;
  r.q = sf64::div_opt(a, b, r.rare);
  return r;
}
// A sum on the integer pipe (correctly rounded; rare operands inside go to the
// hardware instruction), for a kernel whose FP64 pipe is the busier one.
__device__ __noinline__ double add_call(double a, double b) { return sf64::add(a, b); }

// Products and quotients of one unit of work: on the integer pipes, noting
// any operand they leave to the hardware ...
struct arith_opt {
  unsigned rare = 0;
  __device__ __forceinline__ double mul(double a, double b) {
    const flagged r = mul_call(a, b);
    rare |= r.rare;
    return r.q;
  }
  __device__ __forceinline__ double quo(double a, double b) {
    const flagged r = div_call(a, b);
    rare |= r.rare;
    return r.q;
  }
  // x * 0.5 and x / 2, the same correctly rounded value: exact while the
  // half is a normal number, so the exponent field drops by one; zeros keep
  // their bits; tiny, infinite and NaN operands are left to the hardware
  __device__ __forceinline__ double half(double x) {
    unsigned lo, hi;
    sf64::halves(x, lo, hi);
    const unsigned e = sf64::expo(hi);
    rare |= (unsigned)((e <= 1u) & !sf64::is_zero(lo, hi)) | (unsigned)(e == 0x7ffu);
    return e > 1u ? sf64::join(lo, hi - (1u << 20)) : x;
  }
};
// ... and with the FP64 instructions (the evaluation kept when `rare`)
struct arith_hw {
  __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  __device__ __forceinline__ double quo(double a, double b) { return __ddiv_rn(a, b); }
  __device__ __forceinline__ double half(double x) { return __dmul_rn(x, 0.5); }
};

// Products of a part of a unit's work on the FP64 pipe (the same correctly
// rounded bits), the rest of the arithmetic as the unit's policy does it: a
// kernel whose integer pipe is the busier one moves some products back.  In
// the fluxes kernel (ALU 79 %, FP64 54 % with every product on the integer
// pipe) the physical flux of one side and the area scaling take the FP64
// pipe: 2D step 1.573 -> 1.521 ms (with the reconstruction of the right side
// as well: 1.572, the FP64 pipe then the busier one).  In dt the dot
// products (1.573 -> 1.568).
template <class A>
struct fp64_products {
  A &ar;
  __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  __device__ __forceinline__ double quo(double a, double b) { return ar.quo(a, b); }
  __device__ __forceinline__ double half(double x) { return ar.half(x); }
};

// IEEE comparisons decided on the integer pipe (an FP64 compare would take an
// FP64 issue slot): order keys of the two's-complement kind, NaN unordered.
__device__ __forceinline__ bool is_nan(unsigned lo, unsigned hi) {
  const unsigned h = hi & 0x7fffffffu;
  return h > 0x7ff00000u || (h == 0x7ff00000u && lo != 0u);
}
__device__ __forceinline__ long long cmp_key(unsigned lo, unsigned hi) {
  // -0 and +0 share a key; a < b exactly when key(a) < key(b) for non-NaN
  long long b = (long long)(((unsigned long long)hi << 32) | lo);
  b = (b == (long long)0x8000000000000000ull) ? 0ll : b;
  return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
// a < b
__device__ __forceinline__ bool lt(double a, double b) {
  unsigned al, ah, bl, bh;
  sf64::halves(a, al, ah);
  sf64::halves(b, bl, bh);
  return !is_nan(al, ah) && !is_nan(bl, bh) && cmp_key(al, ah) < cmp_key(bl, bh);
}
// x >= 0, x <= 0, x < 0
__device__ __forceinline__ bool ge0(double x) {
  unsigned lo, hi;
  sf64::halves(x, lo, hi);
  return !is_nan(lo, hi) && ((hi >> 31) == 0u || sf64::is_zero(lo, hi));
}
__device__ __forceinline__ bool le0(double x) {
  unsigned lo, hi;
  sf64::halves(x, lo, hi);
  return !is_nan(lo, hi) && ((hi >> 31) != 0u || sf64::is_zero(lo, hi));
}
__device__ __forceinline__ bool lt0(double x) {
  unsigned lo, hi;
  sf64::halves(x, lo, hi);
  return !is_nan(lo, hi) && (hi >> 31) != 0u && !sf64::is_zero(lo, hi);
}
// x == +-0
__device__ __forceinline__ bool is_zero(double x) {
  unsigned lo, hi;
  sf64::halves(x, lo, hi);
  return sf64::is_zero(lo, hi);
}
// neither -0 nor a NaN (x + (+-0) == x bit for bit)
__device__ __forceinline__ bool ordinary(double x) {
  unsigned lo, hi;
  sf64::halves(x, lo, hi);
  return !is_nan(lo, hi) && !(hi == 0x80000000u && lo == 0u);
}
// |x| by clearing the sign bit
__device__ __forceinline__ double absval(double x) {
  unsigned lo, hi;
  sf64::halves(x, lo, hi);
  return sf64::join(lo, hi & 0x7fffffffu);
}

// std::max / std::min semantics of the reference (a < b ? b : a)
__device__ __forceinline__ double smax(double a, double b) { return lt(a, b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return lt(b, a) ? b : a; }

template <int D, class A>
__device__ __forceinline__ double dot(A &ar, const double *a, const double *b) {
  double s = 0;
#pragma unroll
  for (int i = 0; i < D; ++i) s += ar.mul(a[i], b[i]);
  return s;
}

// Same slots as pack_copy(c, d, v, p, e, T, a) (tasks.h:420).  T is carried by
// the reference but never used in a flux, so it is not loaded here.
template <int D>
struct prim {
  double d, v[D], p, e, a;
};

template <int D, class A>
__device__ __forceinline__ double total_energy(A &ar, const prim<D> &u) {
  return u.e + ar.half(dot<D>(ar, u.v, u.v));  // 0.5 * |v|^2
}

template <int D, class A>
__device__ __forceinline__ void phys_flux(A &ar, const prim<D> &u, const double *n, double *f) {
  const double et = total_energy<D>(ar, u);
  const double vn = dot<D>(ar, u.v, n);
  const double mass_flux = ar.mul(u.d, vn);
  f[0] = mass_flux;
#pragma unroll
  for (int i = 0; i < D; ++i) f[1 + i] = ar.mul(mass_flux, u.v[i]) + ar.mul(u.p, n[i]);
  f[D + 1] = ar.mul(mass_flux, et + ar.quo(u.p, u.d));
}

template <int D, class A>
__device__ __forceinline__ void solution_delta(A &ar, const prim<D> &l, const prim<D> &r,
                                               double *du) {
  const double ener_l = ar.mul(l.d, total_energy<D>(ar, l));
  const double ener_r = ar.mul(r.d, total_energy<D>(ar, r));
  du[0] = r.d - l.d;
#pragma unroll
  for (int i = 0; i < D; ++i) du[1 + i] = ar.mul(r.d, r.v[i]) - ar.mul(l.d, l.v[i]);
  du[D + 1] = ener_r - ener_l;
}

template <int D, class A>
__device__ __forceinline__ void hlle(A &ar, const prim<D> &l, const prim<D> &r,
                                     const double *n, double *f) {
  const double vnl = dot<D>(ar, l.v, n), vnr = dot<D>(ar, r.v, n);
  const double lambda_l = smin(vnl - l.a, vnr - r.a);
  const double lambda_r = smax(vnl + l.a, vnr + r.a);
  // one physical-flux evaluation per side: the upwind side's (or the left
  // side's when both are needed), then the right side's if both are
  const bool up_l = ge0(lambda_l), up_r = !up_l && le0(lambda_r);
  phys_flux<D>(ar, up_r ? r : l, n, f);
  if (up_l || up_r) return;
  double fr[D + 2], du[D + 2];
  phys_flux<D>(ar, r, n, fr);
  const double c1 = ar.mul(lambda_l, lambda_r);
  const double c2 = lambda_r - lambda_l;
  const double c2inv = ar.quo(1, c2);
  solution_delta<D>(ar, l, r, du);
#pragma unroll
  for (int i = 0; i < D + 2; ++i)
    f[i] = ar.mul(c2inv, ar.mul(lambda_r, f[i]) - ar.mul(lambda_l, fr[i]) + ar.mul(c1, du[i]));
}

template <int D, class A>
__device__ __forceinline__ void rusanov(A &ar, const prim<D> &l, const prim<D> &r,
                                        const double *n, double *f) {
  double fl[D + 2], fr[D + 2], du[D + 2];
  {
    fp64_products<A> pp{ar};
    phys_flux<D>(pp, l, n, fl);
  }
  phys_flux<D>(ar, r, n, fr);
  const double sl = l.a + absval(dot<D>(ar, l.v, n));
  const double sr = r.a + absval(dot<D>(ar, r.v, n));
  const double s = smax(sl, sr);
  solution_delta<D>(ar, l, r, du);
  const double half_s = ar.half(s);  // s / 2
#pragma unroll
  for (int i = 0; i < D + 2; ++i) f[i] = ar.half(fl[i] + fr[i]) - ar.mul(du[i], half_s);
}

// Toro's HLLC (sec. 10.4) with the hlle_flux wave-speed estimates.
template <int D, class A>
__device__ __forceinline__ void hllc(A &ar, const prim<D> &l, const prim<D> &r,
                                     const double *n, double *f) {
  const double vnl = dot<D>(ar, l.v, n), vnr = dot<D>(ar, r.v, n);
  const double sL = smin(vnl - l.a, vnr - r.a);
  const double sR = smax(vnl + l.a, vnr + r.a);
  // one physical-flux evaluation: of the upwind side, or of the star
  // region's side, which then takes its correction
  const bool up_l = ge0(sL), up_r = !up_l && le0(sR), star = !(up_l || up_r);
  double ml = 0, mr = 0, sM = 0;
  bool left = up_l;
  if (star) {
    ml = ar.mul(l.d, sL - vnl);
    mr = ar.mul(r.d, sR - vnr);
    sM = ar.quo(r.p - l.p + ar.mul(ml, vnl) - ar.mul(mr, vnr), ml - mr);
    left = ge0(sM);
  }
  const prim<D> &u = left ? l : r;
  {
    fp64_products<A> pp{ar};
    phys_flux<D>(pp, u, n, f);
  }
  if (!star) return;
  const double sK = left ? sL : sR;
  const double mK = left ? ml : mr;
  const double vnK = left ? vnl : vnr;
  const double EK = ar.mul(u.d, total_energy<D>(ar, u));
  const double fac = ar.quo(mK, sK - sM);
  const double dvn = sM - vnK;
  f[0] = f[0] + ar.mul(sK, fac - u.d);
#pragma unroll
  for (int i = 0; i < D; ++i)
    f[1 + i] = f[1 + i] +
               ar.mul(sK, ar.mul(fac, u.v[i] + ar.mul(dvn, n[i])) - ar.mul(u.d, u.v[i]));
  f[D + 1] = f[D + 1] +
             ar.mul(sK, ar.mul(fac, ar.quo(EK, u.d) + ar.mul(dvn, sM + ar.quo(u.p, mK))) - EK);
}

// ---------------------------------------------------------------------------
// Order-preserving integer keys of doubles.  Minima and maxima of doubles run
// on the integer pipe through these keys.  key(a) < key(b) exactly when a < b
// for non-NaN values; -0 and +0 share the key of +0, so a minimum or maximum
// can differ from the floating-point one only in the sign of a zero.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long okey(double x) {
  long long b = __double_as_longlong(x);
  b = (b == (long long)0x8000000000000000ull) ? 0ll : b;
  return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
__device__ __forceinline__ double from_okey(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffll));
}

// ---------------------------------------------------------------------------
// dt: per-block maxima of (a + |v.n|) / (V/A), then one block finishes.
// With PRE the V/A of each (cell, face) slot comes from a table built once per
// mesh by the same division.
// ---------------------------------------------------------------------------
template <int D, bool PRE, class A>
__device__ __forceinline__ double cell_dt_inv(A &ar, const fvh_mesh_view &m,
                                              const fvh_state_view &s, int c,
                                              const double *__restrict__ slot_dx) {
  double v[D];
#pragma unroll
  for (int i = 0; i < D; ++i) v[i] = s.velocity[i][c];
  const double a = s.sound_speed[c];
  const double vol = PRE ? 0.0 : m.cell_volume[c];
  double dt_inv = 0;
  const int q0 = m.cell_face_offsets[c], q1 = m.cell_face_offsets[c + 1];
  for (int q = q0; q < q1; ++q) {
    int f = m.cell_faces[q];
    f = f < 0 ? ~f : f;
    double n[D];
#pragma unroll
    for (int i = 0; i < D; ++i) n[i] = m.face_normal[i][f];
    const double delta_x = PRE ? slot_dx[q] : ar.quo(vol, m.face_area[f]);
    fp64_products<A> pp{ar};
    const double dti = ar.quo(a + absval(dot<D>(pp, v, n)), delta_x);
    dt_inv = smax(dti, dt_inv);
  }
  return dt_inv;
}

// With has_src the state is read from src (e.g. host-mapped planes of a caller
// that holds its state in host memory) and stored into s as it goes, all but
// the temperature, which no kernel of the step reads.
template <int D, bool PRE>
__global__ void __launch_bounds__(kDtThreads)
dt_partial_kernel(const fvh_mesh_view m, const fvh_state_view s, double *partial,
                  const double *__restrict__ slot_dx, const fvh_state_view src, int has_src) {
  double dt_inv = 0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.num_cells;
       c += gridDim.x * blockDim.x) {
    if (has_src) {
      s.density[c] = src.density[c];
#pragma unroll
      for (int i = 0; i < D; ++i) s.velocity[i][c] = src.velocity[i][c];
      s.internal_energy[c] = src.internal_energy[c];
      s.pressure[c] = src.pressure[c];
      s.sound_speed[c] = src.sound_speed[c];
    }
    arith_opt ar;
    double cell = cell_dt_inv<D, PRE>(ar, m, s, c, slot_dx);
    if (ar.rare) {
      arith_hw hw;
      cell = cell_dt_inv<D, PRE>(hw, m, s, c, slot_dx);
    }
    // the reference's running maximum over cells and faces, taken cell by
    // cell (a maximum of maxima: the same value)
    dt_inv = smax(cell, dt_inv);
  }
  dt_inv = block_max(dt_inv);
  if (threadIdx.x == 0) partial[blockIdx.x] = dt_inv;
}

__global__ void __launch_bounds__(kDtThreads)
dt_final_kernel(const double *partial, int nblocks, fvh_params p,
                const double *soln_time, double *dt_out, fvh_device_status *status) {
  double dt_inv = 0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) dt_inv = smax(partial[i], dt_inv);
  dt_inv = block_max(dt_inv);
  if (threadIdx.x == 0) {
    const double max_dt = p.final_time - soln_time[0];
    if (le0(dt_inv)) {
      atomicMin(status, status_key(0, FVH_ERR_INFINITE_DT));
      dt_out[0] = 0;
    } else {
      double time_step = __ddiv_rn(1, dt_inv);
      time_step = __dmul_rn(time_step, p.cfl);
      dt_out[0] = smin(time_step, max_dt);
    }
  }
}

// ---------------------------------------------------------------------------
// Geometry-only tables built once per mesh for the solver (same operations in
// the same order as the on-the-fly code, so the values are identical).
// ---------------------------------------------------------------------------
// lsq record per cell: 2D (a00 a01 a11 denom); 3D (a00 a01 a02 a11 a12 a22
// min1 min2 min3 denom), tasks.h:210-228 and :250-261
template <int D>
struct lsq_width {
  static constexpr int value = D == 2 ? 4 : 10;
};

template <int D, class A>
__device__ __forceinline__ void lsq_matrix(A &ar, const fvh_mesh_view &m, int c0, double *r) {
  double x0[D];
#pragma unroll
  for (int i = 0; i < D; ++i) x0[i] = m.cell_centroid[i][c0];
  double dxdx[6] = {0, 0, 0, 0, 0, 0};
  for (int q = m.cell_nbr_offsets[c0]; q < m.cell_nbr_offsets[c0 + 1]; ++q) {
    const int c1 = m.cell_nbrs[q];
    double dx[D];
#pragma unroll
    for (int d = 0; d < D; ++d) dx[d] = m.cell_centroid[d][c1] - x0[d];
    if (D == 2) {
      dxdx[0] += ar.mul(dx[0], dx[0]);
      dxdx[1] += ar.mul(dx[0], dx[1]);
      dxdx[2] += ar.mul(dx[1], dx[1]);
    } else {
      dxdx[0] += ar.mul(dx[0], dx[0]);
      dxdx[1] += ar.mul(dx[0], dx[1]);
      dxdx[2] += ar.mul(dx[0], dx[D - 1]);
      dxdx[3] += ar.mul(dx[1], dx[1]);
      dxdx[4] += ar.mul(dx[1], dx[D - 1]);
      dxdx[5] += ar.mul(dx[D - 1], dx[D - 1]);
    }
  }
  if (D == 2) {
    r[0] = dxdx[0];
    r[1] = dxdx[1];
    r[2] = dxdx[2];
    r[3] = ar.quo(1, ar.mul(dxdx[0], dxdx[2]) - ar.mul(dxdx[1], dxdx[1]));
  } else {
    const double a00 = dxdx[0], a01 = dxdx[1], a02 = dxdx[2], a11 = dxdx[3],
                 a12 = dxdx[4], a22 = dxdx[5];
    const double min1 = ar.mul(a11, a22) - ar.mul(a12, a12);
    const double min2 = ar.mul(a01, a22) - ar.mul(a12, a02);
    const double min3 = ar.mul(a01, a12) - ar.mul(a11, a02);
    for (int k = 0; k < 6; ++k) r[k] = dxdx[k];
    r[6] = min1;
    r[7] = min2;
    r[8] = min3;
    r[9] = ar.quo(1, ar.mul(a00, min1) - ar.mul(a01, min2) + ar.mul(a02, min3));
  }
}

template <int D>
__global__ void cell_tables_kernel(const fvh_mesh_view m, double *lsq, double *slot_dx,
                                   double *nbr_dx, double *vtx_dx) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.num_cells) return;
  arith_hw hw;  // set-up, once per mesh
  constexpr int W = lsq_width<D>::value;
  double r[W];
  lsq_matrix<D>(hw, m, c, r);
#pragma unroll
  for (int k = 0; k < W; ++k) lsq[(size_t)k * m.num_cells + c] = r[k];
  const double vol = m.cell_volume[c];
  for (int q = m.cell_face_offsets[c]; q < m.cell_face_offsets[c + 1]; ++q) {
    int f = m.cell_faces[q];
    f = f < 0 ? ~f : f;
    slot_dx[q] = hw.quo(vol, m.face_area[f]);
  }
  double x0[D];
#pragma unroll
  for (int i = 0; i < D; ++i) x0[i] = m.cell_centroid[i][c];
  for (int q = m.cell_nbr_offsets[c]; q < m.cell_nbr_offsets[c + 1]; ++q) {
    const int c1 = m.cell_nbrs[q];
#pragma unroll
    for (int d = 0; d < D; ++d) nbr_dx[(size_t)q * D + d] = m.cell_centroid[d][c1] - x0[d];
  }
  for (int q = m.cell_vertex_offsets[c]; q < m.cell_vertex_offsets[c + 1]; ++q) {
    const int v = m.cell_vertices[q];
#pragma unroll
    for (int d = 0; d < D; ++d) vtx_dx[(size_t)q * D + d] = m.vertex_coord[d][v] - x0[d];
  }
}

template <int D>
__global__ void face_tables_kernel(const fvh_mesh_view m, double *face_dx) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.num_faces) return;
  const int2 cc = reinterpret_cast<const int2 *>(m.face_cells)[f];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const int c = side == 0 ? cc.x : cc.y;
#pragma unroll
    for (int i = 0; i < D; ++i)
      face_dx[(size_t)f * 2 * D + side * D + i] =
          c >= 0 ? m.face_centroid[i][f] - m.cell_centroid[i][c] : 0.0;
  }
}

// ---------------------------------------------------------------------------
// gradients + Barth-Jespersen vertex limiter (tasks.h:145-321)
// With PRE the geometry-only terms (matrix, neighbour and vertex offsets) come
// from the solver's tables.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void load_dx(const double *__restrict__ p, double *dx) {
  if (D == 2) {
    const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    dx[0] = v.x;
    dx[D - 1] = v.y;
  } else {
#pragma unroll
    for (int d = 0; d < D; ++d) dx[d] = __ldg(p + d);
  }
}

// Plane k of the reconstructed variables (d, v.., e, p, a) of a state and of
// its gradients (component i).
template <int D>
__device__ __forceinline__ const double *state_plane(const fvh_state_view &s, int k) {
  return k == 0 ? s.density
                : k <= D ? s.velocity[k - 1]
                         : k == D + 1 ? s.internal_energy
                                      : k == D + 2 ? s.pressure : s.sound_speed;
}
template <int D>
__device__ __forceinline__ double *grad_plane(const fvh_gradient_view &g, int k, int i) {
  return k == 0 ? g.density[i]
                : k <= D ? g.velocity[k - 1][i]
                         : k == D + 1 ? g.internal_energy[i]
                                      : k == D + 2 ? g.pressure[i] : g.sound_speed[i];
}

template <int D, int K0, int NK>
__device__ __forceinline__ void load_values(const fvh_state_view &s, int c, double *u) {
#pragma unroll
  for (int k = 0; k < NK; ++k) u[k] = state_plane<D>(s, K0 + k)[c];
}

// The limited gradients gu of cell c0 for the reconstructed variables
// K0 .. K0+NK-1 (of d, v.., e, p, a).  Each variable's gradient and limiter
// depend on that variable alone, so the variables can be taken in groups, each
// in its own pass over the neighbours (fewer live registers, same results).
template <int D, int K0, int NK, bool LIMIT, bool PRE, class A>
__device__ __forceinline__ void cell_gradients(A &ar, const fvh_mesh_view &m,
                                               const fvh_state_view &s, const tables &t,
                                               int c0, double (&gu)[NK][D]) {
  constexpr int NV = NK;
  constexpr int W = lsq_width<D>::value;
  constexpr double tol = 1.e-9;
  double x0[D];
  if (!PRE) {
#pragma unroll
    for (int i = 0; i < D; ++i) x0[i] = m.cell_centroid[i][c0];
  }
  double u0[NV];
  load_values<D, K0, NK>(s, c0, u0);
  double dudx[NV][D];
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int j = 0; j < D; ++j) dudx[k][j] = 0;
  const int q0 = m.cell_nbr_offsets[c0], q1 = m.cell_nbr_offsets[c0 + 1];
  #pragma unroll 1
  for (int q = q0; q < q1; ++q) {
    const int c1 = m.cell_nbrs[q];
    double u1[NV];
    load_values<D, K0, NK>(s, c1, u1);
    double dx[D];
    if (PRE) {
      load_dx<D>(t.nbr_dx + (size_t)q * D, dx);
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) dx[d] = m.cell_centroid[d][c1] - x0[d];
    }
    double du[NV];
    unsigned nonzero = 0;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      du[k] = u1[k] - u0[k];
      nonzero |= (unsigned)!is_zero(du[k]);
    }
    // a neighbour equal to the cell in every variable adds (+-0) * dx = +-0 to
    // each sum, which leaves it as it is (a sum that starts at +0 and adds
    // nonzero terms is never -0): cells inside a uniform region skip it
    if (nonzero) {
#pragma unroll
      for (int k = 0; k < NV; ++k)
#pragma unroll
        for (int j = 0; j < D; ++j) dudx[k][j] += ar.mul(du[k], dx[j]);
    }
  }
  double r[W];
  if (PRE) {
#pragma unroll
    for (int k = 0; k < W; ++k) r[k] = t.lsq[(size_t)k * m.num_cells + c0];
  } else {
    lsq_matrix<D>(ar, m, c0, r);
  }
  if (D == 2) {
    const double a00 = r[0], a01 = r[1], a11 = r[2], denom = r[3];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      gu[k][0] = ar.mul(ar.mul(dudx[k][0], a11) - ar.mul(dudx[k][1], a01), denom);
      gu[k][D - 1] = ar.mul(ar.mul(dudx[k][1], a00) - ar.mul(dudx[k][0], a01), denom);
    }
  } else {
    const double a00 = r[0], a01 = r[1], a02 = r[2], a11 = r[3], a12 = r[4], a22 = r[5];
    const double min1 = r[6], min2 = r[7], min3 = r[W - 2], denom = r[W - 1];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double b0 = dudx[k][0], b1 = dudx[k][1], b2 = dudx[k][D - 1];
      gu[k][0] = ar.mul(ar.mul(b0, min1) - ar.mul(a01, ar.mul(b1, a22) - ar.mul(a12, b2)) +
                            ar.mul(a02, ar.mul(b1, a12) - ar.mul(a11, b2)),
                        denom);
      gu[k][1] = ar.mul(ar.mul(a00, ar.mul(b1, a22) - ar.mul(a12, b2)) - ar.mul(b0, min2) +
                            ar.mul(a02, ar.mul(b2, a01) - ar.mul(a02, b1)),
                        denom);
      gu[k][D - 1] = ar.mul(ar.mul(a00, ar.mul(b2, a11) - ar.mul(a12, b1)) -
                                ar.mul(a01, ar.mul(b2, a01) - ar.mul(a02, b1)) +
                                ar.mul(b0, min3),
                            denom);
    }
  }
  if (LIMIT) {
    // phi_k = min over vertices of (umax-u0)/du or (umin-u0)/du.  Correctly
    // rounded division is monotone in the divisor, so for each variable only
    // the largest du > tol and the smallest du < -tol can set the minimum; the
    // result equals the reference's per-vertex minimum.
    const long long ktol = okey(tol), kntol = okey(-tol);
    long long kpos[NV], kneg[NV];
    // a variable with a zero gradient has u1 == u0 at every vertex (to the
    // sign of a zero, which the order keys do not see): no vertex limits it
    bool graded[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      kpos[k] = kneg[k] = 0;
      graded[k] = false;
#pragma unroll
      for (int i = 0; i < D; ++i) graded[k] = graded[k] || !is_zero(gu[k][i]);
    }
    const int r0 = m.cell_vertex_offsets[c0], r1 = m.cell_vertex_offsets[c0 + 1];
    #pragma unroll 1
    for (int rr = r0; rr < r1; ++rr) {
      double dxv[D];
      if (PRE) {
        load_dx<D>(t.vtx_dx + (size_t)rr * D, dxv);
      } else {
        const int vtx = m.cell_vertices[rr];
#pragma unroll
        for (int i = 0; i < D; ++i) dxv[i] = m.vertex_coord[i][vtx] - x0[i];
      }
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        if (!graded[k]) continue;
        double u1 = u0[k];
#pragma unroll
        for (int i = 0; i < D; ++i) u1 += ar.mul(dxv[i], gu[k][i]);
        const long long kd = okey(u1 - u0[k]);
        if (kd > ktol) kpos[k] = (kpos[k] < kd) ? kd : kpos[k];
        else if (kd < kntol) kneg[k] = (kd < kneg[k]) ? kd : kneg[k];
      }
    }
    // the neighbour extrema umin / umax (tasks.h:232-236) are needed only for
    // a variable some vertex value departs from by more than tol: they are
    // taken then, in a second pass over the neighbours (whose values are
    // still in cache), as order keys
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      long long kphi = okey(1.0);
      if (kpos[k] > ktol || kneg[k] < kntol) {
        const double *plane = state_plane<D>(s, K0 + k);
        long long kmin = okey(u0[k]), kmax = kmin;
        #pragma unroll 1
        for (int q = q0; q < q1; ++q) {
          const long long k1 = okey(plane[m.cell_nbrs[q]]);
          kmin = (k1 < kmin) ? k1 : kmin;  // std::min(u1, umin)
          kmax = (kmax < k1) ? k1 : kmax;  // std::max(u1, umax)
        }
        // RN(N / du) >= 1 exactly when |N| >= |du| (N and du of one sign, du
        // normal), so the quotient is formed only when it can lower phi below 1
        if (kpos[k] > ktol) {
          const double num = from_okey(kmax) - u0[k];
          if (okey(num) < kpos[k]) {
            const long long kq = okey(ar.quo(num, from_okey(kpos[k])));
            kphi = (kq < kphi) ? kq : kphi;
          }
        }
        if (kneg[k] < kntol) {
          const double num = from_okey(kmin) - u0[k];
          if (okey(num) > kneg[k]) {
            const long long kq = okey(ar.quo(num, from_okey(kneg[k])));
            kphi = (kq < kphi) ? kq : kphi;
          }
        }
      }
      kphi = (kphi < 0) ? 0 : kphi;  // std::max(phi, 0)
      if (kphi != okey(1.0)) {
        const double phi = from_okey(kphi);
#pragma unroll
        for (int i = 0; i < D; ++i) gu[k][i] = ar.mul(gu[k][i], phi);
      }
    }
  }
}

template <int D, int K0, int NK>
__device__ __forceinline__ void store_gradients(const fvh_gradient_view &g, int c0,
                                                const double (&gu)[NK][D]) {
#pragma unroll
  for (int k = 0; k < NK; ++k)
#pragma unroll
    for (int i = 0; i < D; ++i) grad_plane<D>(g, K0 + k, i)[c0] = gu[k][i];
}

// the FP64 redo of a cell whose operands left the integer-pipe range, out of
// line (it is rare and would otherwise double the kernel's code)
template <int D, int K0, int NK, bool LIMIT, bool PRE>
__device__ __noinline__ void gradient_group_hw(const fvh_mesh_view &m, const fvh_state_view &s,
                                               const fvh_gradient_view &g, const tables &t,
                                               int c0) {
  double gu[NK][D];
  arith_hw hw;
  cell_gradients<D, K0, NK, LIMIT, PRE>(hw, m, s, t, c0, gu);
  store_gradients<D, K0, NK>(g, c0, gu);
}

// the gradients of variables K0 .. K0+NK-1 of cell c0, stored
template <int D, int K0, int NK, bool LIMIT, bool PRE>
__device__ __forceinline__ void gradient_group(const fvh_mesh_view &m, const fvh_state_view &s,
                                               const fvh_gradient_view &g, const tables &t,
                                               int c0) {
  double gu[NK][D];
  arith_opt ar;
  cell_gradients<D, K0, NK, LIMIT, PRE>(ar, m, s, t, c0, gu);
  if (ar.rare) {
    gradient_group_hw<D, K0, NK, LIMIT, PRE>(m, s, g, t, c0);
    return;
  }
  store_gradients<D, K0, NK>(g, c0, gu);
}

// Blocks of 128 per SM the kernels are compiled for.  2D (1024^2 workload, ms
// per step): fluxes 7 (72 registers) 1.493 against 1.502 with 6 and 1.542
// with 8; gradients 10 (48 registers, variables in pairs, below) 1.572
// against 1.582 with 8; update 10 (48 registers) 1.487 against 1.502 with
// the compiler's choice (66 registers) and 1.493 with 8.  3D (96^3 hex):
// gradients and fluxes 5 blocks (96 registers) 5.68 against 5.92 with 3 and
// 4 and 5.88 with 4 and 5; update the compiler's choice.
template <int D>
constexpr int min_blocks() { return D == 2 ? 7 : 5; }
template <int D>
constexpr int grad_min_blocks() { return D == 2 ? 10 : 5; }
template <int D>
constexpr int update_min_blocks() { return D == 2 ? 10 : 1; }
// Variables per neighbour pass of the gradients.  Each variable's gradient
// and limiter depend on that variable alone, so the variables can be taken in
// groups, each in its own pass over the neighbours (the neighbours' values
// are re-read, mostly from L1/L2): fewer live sums, more warps.  2D in pairs
// (d vx, vy e, p a): 1.572 ms per step against 1.755 with all six in one pass
// and 1.592 in threes; 3D in groups of four (d v, then e p a): 5.30 against
// 5.58 in threes (6 blocks) and 5.30 in pairs.
template <int D>
__host__ __device__ constexpr int grad_split() { return D == 2 ? 2 : D + 1; }

// the variables K0 .. NV-1 in groups of G, each group in its own pass
template <int D, int K0, int G, bool LIMIT, bool PRE>
__device__ __forceinline__ void gradient_groups(const fvh_mesh_view &m, const fvh_state_view &s,
                                                const fvh_gradient_view &g, const tables &t,
                                                int c0) {
  constexpr int NV = D + 4, NK = (NV - K0 < G) ? NV - K0 : G;
  gradient_group<D, K0, NK, LIMIT, PRE>(m, s, g, t, c0);
  if constexpr (K0 + NK < NV) gradient_groups<D, K0 + NK, G, LIMIT, PRE>(m, s, g, t, c0);
}

template <int D, bool LIMIT, bool PRE>
__global__ void __launch_bounds__(kCellThreads, grad_min_blocks<D>())
gradients_kernel(const fvh_mesh_view m, const fvh_state_view s, const fvh_gradient_view g,
                 const tables t) {
  const int c0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (c0 >= m.num_cells) return;
  gradient_groups<D, 0, grad_split<D>(), LIMIT, PRE>(m, s, g, t, c0);
}

// ---------------------------------------------------------------------------
// face fluxes (tasks.h:385-464)
// ---------------------------------------------------------------------------
template <int D, bool SECOND, class A>
__device__ __forceinline__ prim<D> reconstruct(A &ar, const fvh_state_view &s,
                                               const fvh_gradient_view &g, int c,
                                               const double *dx, bool swap) {
  prim<D> w;
  w.d = s.density[c];
#pragma unroll
  for (int i = 0; i < D; ++i) w.v[i] = s.velocity[i][c];
  w.p = s.pressure[c];
  w.e = s.internal_energy[c];
  w.a = s.sound_speed[c];
  if (SECOND) {
    double *const *gp = swap ? g.internal_energy : g.pressure;
    double *const *ge = swap ? g.pressure : g.internal_energy;
    double gd[D], gv[D][D], gpp[D], gee[D], ga[D];
    unsigned nonzero = 0;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      gd[i] = g.density[i][c];
      nonzero |= (unsigned)!is_zero(gd[i]);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        gv[d][i] = g.velocity[d][i][c];
        nonzero |= (unsigned)!is_zero(gv[d][i]);
      }
      gpp[i] = gp[i][c];
      gee[i] = ge[i][c];
      ga[i] = g.sound_speed[i][c];
      nonzero |= (unsigned)(!is_zero(gpp[i]) | !is_zero(gee[i]) | !is_zero(ga[i]));
    }
    // zero gradients add dx * (+-0) = +-0 to each value (dx is finite), which
    // leaves it as it is unless the value is -0 or a NaN: cells with uniform
    // neighbourhoods skip the products when no value is one of those
    unsigned plain = (unsigned)(ordinary(w.d) & ordinary(w.p) & ordinary(w.e) & ordinary(w.a));
#pragma unroll
    for (int d = 0; d < D; ++d) plain &= (unsigned)ordinary(w.v[d]);
    if (nonzero | !plain) {
#pragma unroll
      for (int i = 0; i < D; ++i) {
        w.d += ar.mul(dx[i], gd[i]);
#pragma unroll
        for (int d = 0; d < D; ++d) w.v[d] += ar.mul(dx[i], gv[d][i]);
        w.p += ar.mul(dx[i], gpp[i]);
        w.e += ar.mul(dx[i], gee[i]);
        w.a += ar.mul(dx[i], ga[i]);
      }
    }
  }
  return w;
}

// x_f - x_c of one side of face f, from the table or on the fly
template <int D, bool PRE>
__device__ __forceinline__ void face_offset(const fvh_mesh_view &m, const double *face_dx,
                                            int f, int side, int c, double *dx) {
  if (PRE) {
    load_dx<D>(face_dx + (size_t)f * 2 * D + side * D, dx);
  } else {
#pragma unroll
    for (int i = 0; i < D; ++i) dx[i] = m.face_centroid[i][f] - m.cell_centroid[i][c];
  }
}

// the area-weighted flux of face f (tasks.h:405-461)
template <int D, int KIND, bool SECOND, bool PRE, class A>
__device__ __forceinline__ void face_flux(A &ar, const fvh_mesh_view &m,
                                          const fvh_state_view &s, const fvh_gradient_view &g,
                                          int f, int2 cc, bool swap, bool outflow,
                                          const double *face_dx, double *F) {
  double n[D];
#pragma unroll
  for (int i = 0; i < D; ++i) n[i] = m.face_normal[i][f];
  double dx[D] = {};
  if (SECOND) face_offset<D, PRE>(m, face_dx, f, 0, cc.x, dx);
  const prim<D> wl = reconstruct<D, SECOND>(ar, s, g, cc.x, dx, swap);
  if (cc.y >= 0) {
    if (SECOND) face_offset<D, PRE>(m, face_dx, f, 1, cc.y, dx);
    const prim<D> wr = reconstruct<D, SECOND>(ar, s, g, cc.y, dx, swap);
    if (KIND == FVH_FLUX_RUSANOV)
      rusanov<D>(ar, wl, wr, n, F);
    else if (KIND == FVH_FLUX_HLLC)
      hllc<D>(ar, wl, wr, n, F);
    else
      hlle<D>(ar, wl, wr, n, F);
  } else if (outflow) {
    phys_flux<D>(ar, wl, n, F);
  } else {
    F[0] = 0;
#pragma unroll
    for (int i = 0; i < D; ++i) F[1 + i] = ar.mul(wl.p, n[i]);
    F[D + 1] = 0;
  }
  const double area = m.face_area[f];
#pragma unroll
  for (int k = 0; k < D + 2; ++k) F[k] = __dmul_rn(F[k], area);
}

// the FP64 redo of a face whose operands left the integer-pipe range, out of
// line
template <int D, int KIND, bool SECOND, bool PRE>
__device__ __noinline__ void face_flux_hw(const fvh_mesh_view &m, const fvh_state_view &s,
                                          const fvh_gradient_view &g, const fvh_flux_view &fl,
                                          int f, int2 cc, int swap, int outflow,
                                          const double *face_dx) {
  double F[D + 2];
  arith_hw hw;
  face_flux<D, KIND, SECOND, PRE>(hw, m, s, g, f, cc, swap != 0, outflow != 0, face_dx, F);
  fl.mass[f] = F[0];
#pragma unroll
  for (int i = 0; i < D; ++i) fl.momentum[i][f] = F[1 + i];
  fl.energy[f] = F[D + 1];
}

template <int D, int KIND, bool SECOND, bool PRE>
__global__ void __launch_bounds__(kFaceThreads, min_blocks<D>())
fluxes_kernel(const fvh_mesh_view m, const fvh_state_view s, const fvh_gradient_view g,
              const fvh_flux_view fl, int swap, int outflow, const double *__restrict__ face_dx) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.num_faces) return;
  const int2 cc = reinterpret_cast<const int2 *>(m.face_cells)[f];
  double F[D + 2];
  {
    arith_opt ar;
    face_flux<D, KIND, SECOND, PRE>(ar, m, s, g, f, cc, swap != 0, outflow != 0, face_dx, F);
    if (ar.rare) {
      face_flux_hw<D, KIND, SECOND, PRE>(m, s, g, fl, f, cc, swap, outflow, face_dx);
      return;
    }
  }
  fl.mass[f] = F[0];
#pragma unroll
  for (int i = 0; i < D; ++i) fl.momentum[i][f] = F[1 + i];
  fl.energy[f] = F[D + 1];
}

// ---------------------------------------------------------------------------
// gather + conservative update + EOS (tasks.h:589-659)
// ---------------------------------------------------------------------------
// the new state of cell c: w = (d, v.., e, p, T, a^2)
// gm1 = gamma - 1 and ggm1 = gamma * (gamma - 1), rounded once on the host
// exactly as the reference rounds them per cell (euler_eqns.h / ideal_gas.h)
template <int D, class A>
__device__ __forceinline__ void cell_update(A &ar, const fvh_mesh_view &m,
                                            const fvh_flux_view &fl, const fvh_state_view &s,
                                            int c, double delta_t, double gm1, double ggm1,
                                            double cv, double *w) {
  double du[D + 2];
#pragma unroll
  for (int k = 0; k < D + 2; ++k) du[k] = 0;
  const int q0 = m.cell_face_offsets[c], q1 = m.cell_face_offsets[c + 1];
  for (int q = q0; q < q1; ++q) {
    const int sf = m.cell_faces[q];
    const int f = sf < 0 ? ~sf : sf;
    double F[D + 2];
    F[0] = fl.mass[f];
#pragma unroll
    for (int i = 0; i < D; ++i) F[1 + i] = fl.momentum[i][f];
    F[D + 1] = fl.energy[f];
    // the update kernel's FP64 pipe is its bound (83 %, ALU 43 %): the sums of
    // the first two faces run on the integer pipe (2D step 1.516 -> 1.488 ms);
    // a - b is a + (-b) exactly
    if (q - q0 < 2) {
      if (sf >= 0) {
#pragma unroll
        for (int k = 0; k < D + 2; ++k) du[k] = add_call(du[k], -F[k]);
      } else {
#pragma unroll
        for (int k = 0; k < D + 2; ++k) du[k] = add_call(du[k], F[k]);
      }
      continue;
    }
    if (sf >= 0) {
#pragma unroll
      for (int k = 0; k < D + 2; ++k) du[k] -= F[k];
    } else {
#pragma unroll
      for (int k = 0; k < D + 2; ++k) du[k] += F[k];
    }
  }
  const double scale = ar.quo(delta_t, m.cell_volume[c]);
#pragma unroll
  for (int k = 0; k < D + 2; ++k) du[k] = ar.mul(du[k], scale);
  double vel[D];
#pragma unroll
  for (int i = 0; i < D; ++i) vel[i] = s.velocity[i][c];
  const double den0 = s.density[c];
  const double mass = den0 + du[0];
  const double ener =
      ar.mul(den0, s.internal_energy[c] + ar.half(dot<D>(ar, vel, vel))) + du[D + 1];
  const double inv_mass = ar.quo(1, mass);
#pragma unroll
  for (int i = 0; i < D; ++i) vel[i] = ar.mul(ar.mul(den0, vel[i]) + du[1 + i], inv_mass);
  const double e = ar.mul(ener, inv_mass) - ar.half(dot<D>(ar, vel, vel));
  w[0] = mass;
#pragma unroll
  for (int i = 0; i < D; ++i) w[1 + i] = vel[i];
  w[D + 1] = e;
  w[D + 2] = ar.mul(ar.mul(gm1, mass), e);
  w[D + 3] = cv == 1.0 ? e : ar.quo(e, cv);  // x / 1 == x exactly
  w[D + 4] = ar.mul(ggm1, e);                 // a^2; its root is taken once
}

template <int D>
__global__ void __launch_bounds__(kCellThreads, update_min_blocks<D>())
update_kernel(const fvh_mesh_view m, const fvh_flux_view fl, const fvh_state_view s,
              const double *dt, double factor, double gm1, double ggm1, double cv,
              double *soln_time, fvh_device_status *status, const fvh_state_view out,
              int has_out) {
  const double delta_t = __dmul_rn(dt[0], factor);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c == 0) soln_time[0] = 0.0 + soln_time[0] + delta_t;
  if (c >= m.num_cells) return;
  double w[D + 5];
  {
    arith_opt ar;
    cell_update<D>(ar, m, fl, s, c, delta_t, gm1, ggm1, cv, w);
    if (ar.rare) {
      arith_hw hw;
      cell_update<D>(hw, m, fl, s, c, delta_t, gm1, ggm1, cv, w);
    }
  }
  const double a = sqrt(w[D + 4]);
  s.density[c] = w[0];
#pragma unroll
  for (int i = 0; i < D; ++i) s.velocity[i][c] = w[1 + i];
  s.internal_energy[c] = w[D + 1];
  s.pressure[c] = w[D + 2];
  s.temperature[c] = w[D + 3];
  s.sound_speed[c] = a;
  if (has_out) {
    out.density[c] = w[0];
#pragma unroll
    for (int i = 0; i < D; ++i) out.velocity[i][c] = w[1 + i];
    out.internal_energy[c] = w[D + 1];
    out.pressure[c] = w[D + 2];
    out.temperature[c] = w[D + 3];
    out.sound_speed[c] = a;
  }
  if (lt0(w[D + 1]) || lt0(w[0])) atomicMin(status, status_key(c, FVH_ERR_NEGATIVE_STATE));
}

// ---------------------------------------------------------------------------
// the integer-pipe arithmetic against the FP64 instructions (diagnostic)
// ---------------------------------------------------------------------------
__global__ void sf64_kernel(int op, const double *a, const double *b, int64_t n, double *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = a[i], y = b[i];
    double r;
    unsigned rare = 0;
    switch (op) {
      case 0: r = sf64::mul(x, y); break;
      case 1: r = sf64::add(x, y); break;
      case 2: r = sf64::sub(x, y); break;
      case 3: r = sf64::div(x, y); break;
      case 4: r = __dmul_rn(x, y); break;
      case 5: r = __dadd_rn(x, y); break;
      case 6: r = __dsub_rn(x, y); break;
      case 7: r = __ddiv_rn(x, y); break;
      case 8:  // the optimistic forms with their redo, as the kernels use them
        r = sf64::mul_opt(x, y, rare);
        if (rare) r = __dmul_rn(x, y);
        break;
      case 10: {  // the kernels' halving of x (0.5 * x and x / 2), with its redo
        arith_opt ar;
        r = ar.half(x);
        if (ar.rare) r = __dmul_rn(x, 0.5);
        break;
      }
      default:
        r = sf64::div_opt(x, y, rare);
        if (rare) r = __ddiv_rn(x, y);
        break;
    }
    out[i] = r;
  }
}

cudaError_t debug_sf64(int op, const double *a, const double *b, int64_t n, double *out,
                       cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int64_t nb64 = (n + 255) / 256;
  const int nb = (int)(nb64 < 4096 ? nb64 : 4096);
  sf64_kernel<<<nb, 256, 0, st>>>(op, a, b, n, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template <int D>
cudaError_t launch_dt(const fvh_mesh_view &m, const fvh_state_view &s,
                      const fvh_params &p, const double *soln_time, double *dt,
                      double *partial, int nblocks, fvh_device_status *status,
                      cudaStream_t st, const double *slot_dx, const fvh_state_view *src) {
  const fvh_state_view from = src ? *src : s;
  if (slot_dx)
    dt_partial_kernel<D, true><<<nblocks, kDtThreads, 0, st>>>(m, s, partial, slot_dx, from,
                                                               src ? 1 : 0);
  else
    dt_partial_kernel<D, false><<<nblocks, kDtThreads, 0, st>>>(m, s, partial, nullptr, from,
                                                                src ? 1 : 0);
  dt_final_kernel<<<1, kDtThreads, 0, st>>>(partial, nblocks, p, soln_time, dt, status);
  return cudaGetLastError();
}

template <int D>
cudaError_t launch_gradients(const fvh_mesh_view &m, const fvh_state_view &s,
                             const fvh_gradient_view &g, const fvh_params &p,
                             cudaStream_t st, const tables &t) {
  const int nb = (m.num_cells + kCellThreads - 1) / kCellThreads;
  const bool lim = p.limiter != FVH_LIMITER_NONE;
  if (t.lsq && t.nbr_dx && t.vtx_dx) {
    if (lim)
      gradients_kernel<D, true, true><<<nb, kCellThreads, 0, st>>>(m, s, g, t);
    else
      gradients_kernel<D, false, true><<<nb, kCellThreads, 0, st>>>(m, s, g, t);
  } else {
    if (lim)
      gradients_kernel<D, true, false><<<nb, kCellThreads, 0, st>>>(m, s, g, t);
    else
      gradients_kernel<D, false, false><<<nb, kCellThreads, 0, st>>>(m, s, g, t);
  }
  return cudaGetLastError();
}

size_t table_doubles(int dim, int64_t nc, int64_t nf, int64_t nnz_cf, int64_t nnz_nb,
                     int64_t nnz_cv) {
  const int64_t w = dim == 2 ? lsq_width<2>::value : lsq_width<3>::value;
  // each table starts on a 256-byte boundary (32 doubles)
  auto up = [](int64_t x) { return (x + 31) / 32 * 32; };
  return (size_t)(up(w * nc) + up(nnz_cf) + up(dim * nnz_nb) + up(dim * nnz_cv) +
                  up(2 * dim * nf));
}

template <int D>
cudaError_t build_tables(const fvh_mesh_view &m, double *base, int64_t nnz_cf,
                         int64_t nnz_nb, int64_t nnz_cv, tables *t) {
  auto up = [](int64_t x) { return (x + 31) / 32 * 32; };
  double *lsq = base;
  double *slot_dx = lsq + up((int64_t)lsq_width<D>::value * m.num_cells);
  double *nbr_dx = slot_dx + up(nnz_cf);
  double *vtx_dx = nbr_dx + up(D * nnz_nb);
  double *face_dx = vtx_dx + up(D * nnz_cv);
  const int th = 128;
  cell_tables_kernel<D><<<(m.num_cells + th - 1) / th, th>>>(m, lsq, slot_dx, nbr_dx, vtx_dx);
  face_tables_kernel<D><<<(m.num_faces + th - 1) / th, th>>>(m, face_dx);
  t->lsq = lsq;
  t->slot_dx = slot_dx;
  t->nbr_dx = nbr_dx;
  t->vtx_dx = vtx_dx;
  t->face_dx = face_dx;
  return cudaGetLastError();
}

template <int D, bool SECOND, bool PRE>
static void launch_fluxes_kind(const fvh_mesh_view &m, const fvh_state_view &s,
                               const fvh_gradient_view &g, const fvh_flux_view &fl,
                               const fvh_params &p, cudaStream_t st, const double *face_dx) {
  const int nb = (m.num_faces + kFaceThreads - 1) / kFaceThreads;
  if (p.flux_kind == FVH_FLUX_RUSANOV)
    fluxes_kernel<D, FVH_FLUX_RUSANOV, SECOND, PRE><<<nb, kFaceThreads, 0, st>>>(
        m, s, g, fl, p.recon_swap_ep, p.boundary, face_dx);
  else if (p.flux_kind == FVH_FLUX_HLLC)
    fluxes_kernel<D, FVH_FLUX_HLLC, SECOND, PRE><<<nb, kFaceThreads, 0, st>>>(
        m, s, g, fl, p.recon_swap_ep, p.boundary, face_dx);
  else
    fluxes_kernel<D, FVH_FLUX_HLLE, SECOND, PRE><<<nb, kFaceThreads, 0, st>>>(
        m, s, g, fl, p.recon_swap_ep, p.boundary, face_dx);
}

template <int D>
cudaError_t launch_fluxes(const fvh_mesh_view &m, const fvh_state_view &s,
                          const fvh_gradient_view &g, const fvh_flux_view &fl,
                          const fvh_params &p, cudaStream_t st, const tables &t) {
  if (p.order == 1)
    launch_fluxes_kind<D, false, false>(m, s, g, fl, p, st, nullptr);
  else if (t.face_dx)
    launch_fluxes_kind<D, true, true>(m, s, g, fl, p, st, t.face_dx);
  else
    launch_fluxes_kind<D, true, false>(m, s, g, fl, p, st, nullptr);
  return cudaGetLastError();
}

template <int D>
cudaError_t launch_update(const fvh_mesh_view &m, const fvh_params &p, const double *dt,
                          double factor, const fvh_flux_view &fl,
                          const fvh_state_view &s, double *soln_time,
                          fvh_device_status *status, cudaStream_t st,
                          const fvh_state_view *out) {
  const int nb = (m.num_cells + kCellThreads - 1) / kCellThreads;
  // the same two roundings as (gamma - 1.0) and gamma * (gamma - 1.0) per cell
  const double gamma = p.gamma;
  const double gm1 = gamma - 1.0;
  const double ggm1 = gamma * gm1;
  update_kernel<D><<<nb, kCellThreads, 0, st>>>(m, fl, s, dt, factor, gm1, ggm1, p.cv,
                                                soln_time, status, out ? *out : s, out ? 1 : 0);
  return cudaGetLastError();
}

#define FVH_INSTANTIATE(D)                                                              \
  template cudaError_t launch_dt<D>(const fvh_mesh_view &, const fvh_state_view &,     \
                                    const fvh_params &, const double *, double *,      \
                                    double *, int, fvh_device_status *, cudaStream_t,  \
                                    const double *, const fvh_state_view *);           \
  template cudaError_t launch_gradients<D>(const fvh_mesh_view &, const fvh_state_view &, \
                                           const fvh_gradient_view &, const fvh_params &, \
                                           cudaStream_t, const tables &);              \
  template cudaError_t build_tables<D>(const fvh_mesh_view &, double *, int64_t, int64_t, \
                                       int64_t, tables *);                             \
  template cudaError_t launch_fluxes<D>(const fvh_mesh_view &, const fvh_state_view &, \
                                        const fvh_gradient_view &, const fvh_flux_view &, \
                                        const fvh_params &, cudaStream_t, const tables &); \
  template cudaError_t launch_update<D>(const fvh_mesh_view &, const fvh_params &,     \
                                        const double *, double, const fvh_flux_view &, \
                                        const fvh_state_view &, double *,              \
                                        fvh_device_status *, cudaStream_t,             \
                                        const fvh_state_view *);
FVH_INSTANTIATE(2)
FVH_INSTANTIATE(3)

}  // namespace plain
}  // namespace fvh
