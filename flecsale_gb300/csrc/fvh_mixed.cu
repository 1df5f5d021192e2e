// Mixed-precision form of the hydro step (sm_103a).
//
// Reconstruction, limiter and Riemann fluxes run in FP32; the cell state stays
// in FP64 and takes its increments in double-float (FP32 pairs, ~48 bits) from
// compensated FP32 face sums; dt is reduced in FP32 and finished in FP64.
// GB300 executes FP64 at 2 operations per clock per SM (FP32: 128), so the
// FP64 pipe is kept to the splits and final additions of the state.  Per time
// step (the structure of apps/hydro/driver.h:325-375):
//
//   pack_dt      FP64 state -> FP32 recon pack (AoS, 32 B/cell); CFL maximum of
//                (a+|v.n|) A/V per block, the last block finishes dt
//                (tasks.h:331-376)
//   gradients    FP32 vertex-neighbour least squares + Barth-Jespersen limiter
//                (tasks.h:145-321), FP32 AoS gradients; in 2D on packed FP32
//                pairs (FFMA2/FADD2/FMUL2)
//   schedule 0:  flux_update: each cell reconstructs both sides of each of its
//                faces, evaluates the Riemann/wall flux in FP32
//                (tasks.h:385-464) and sums -/+F in its face order, then
//                updates (tasks.h:589-659)
//   schedule 1:  face_flux (one flux per face into an array) + gather_update
//                (the same sums in the same order, then the update)
//   schedule 2:  face_colour per colour (fluxes added to both cells' sums) +
//                colour_update
//   predictor update: writes the double-float increments and the FP32 pack of
//                the predicted state, no FP64 state
//   (gradients, fluxes again for the corrector, whose update writes the FP64
//   state = old state + both stages' increments; inside a run it also writes
//   the next step's pack and dt, and that step skips pack_dt)
//
// A face flux has the same bits wherever it is evaluated, so the update is
// conservative to double-float rounding without atomics.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <new>
#include <vector>

#include "fvh_kernels.h"
#include "fvh_mixed.h"
#include "fvh_physics.cuh"
#include "fvh_tma.cuh"

namespace fvh {
namespace mixed {

using phys::prim;
using phys::smax;
using phys::smin;

constexpr int kMaxColours = 32;

// per-cell AoS record sizes in float4 units
template <int D>
struct layout {
  static constexpr int NV = D + 4;             // d, v[D], e, p, a
  static constexpr int PACK4 = 2;              // d v.. p e a (8 floats)
  static constexpr int GRAD4 = D == 2 ? 3 : 6; // NV*D floats, padded
  static constexpr int CEN4 = D == 2 ? 1 : 2;  // centroid hi/lo
  static constexpr int FGEO4 = 1;              // normal[D], area
  static constexpr int FDX4 = D == 2 ? 1 : 2;  // x_f - x_c0, x_f - x_c1
  static constexpr int FLUX4 = D == 2 ? 1 : 2; // face flux (D+2 floats, padded)
  static constexpr int DEL4 = D == 2 ? 2 : 3;  // predictor increments (D+2 double-floats)
};

// Staged 2D gradients (gradients_staged_kernel).  A chunk is a set of up to
// kStageCells cells; its staged records are listed as runs of consecutive ids:
// ids [first, first + count) go to positions [slot, slot + count); kind 0 =
// cells (pack + centroid), 1 = vertices.
struct stage_run {
  int first, count, slot, kind;
};

struct stage_tables {
  int nchunks = 0;
  // layout of one stage buffer (bytes), sized for this mesh's largest chunk:
  // pack records (32 B) at 0, centroids (16 B) at cen_at, vertex coordinates
  // (16 B) at vtx_at, the chunk's topology block at topo_at
  int cen_at = 0, vtx_at = 0, topo_at = 0, stage_bytes = 0;
  const int *cells = nullptr;                // [nchunks * kStageCells] cell ids, -1 = none
  const int *run_off = nullptr;              // [nchunks + 1] into runs
  const stage_run *runs = nullptr;
  const long long *topo_off = nullptr;       // [nchunks + 1] byte offsets into topo
  const unsigned *bytes = nullptr;           // [nchunks] bytes staged per chunk
  const unsigned *topo = nullptr;            // per chunk: see setup_stage_host
};

struct workspace {
  int dim = 0, nc = 0, nf = 0, nv = 0;
  void *base = nullptr;
  float4 *pack = nullptr;    // FP32 recon pack of the predictor (from the FP64 state)
  float4 *pack2 = nullptr;   // pack of the corrector (written by the predictor update)
  float4 *grads = nullptr;
  float4 *ccen = nullptr;    // cell centroid hi/lo
  float4 *vcoord = nullptr;  // vertex coordinates hi/lo
  float4 *fgeo = nullptr;    // face normal + area
  float4 *fdx = nullptr;     // face centroid offsets from both cells
  float4 *fflux = nullptr;   // face schedule: area-scaled face fluxes
  float4 *delta = nullptr;   // predictor increments of (d, v.., e) as double-floats
  float *inv_vol32 = nullptr;  // 1/V rounded to FP32 (CFL estimate; update, high part)
  float *inv_vol_lo = nullptr; // 1/V - inv_vol32, rounded to FP32 (update, low part)
  unsigned *ticket = nullptr;  // blocks done (the last one computes dt)
  unsigned *dtinv_max = nullptr;  // corrector's CFL maximum for the next step (FP32 bits)
  // colour schedule (single mesh): faces grouped by colour, no two faces of a
  // colour share a cell; per-cell compensated face sums (hi[D+2], lo[D+2])
  int *colour_faces = nullptr;
  float *acc = nullptr;
  int ncolours = 0;
  int colour_off[kMaxColours + 1] = {};
  // staged 2D gradients (single mesh, when every chunk fits); stage_base owns
  // the tables' device memory
  stage_tables stage;
  void *stage_base = nullptr;
  int stage_blocks = 0;  // persistent grid
};

__device__ __forceinline__ void stg256(float4 *p, float4 a, float4 b) {
  asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(a.x),
               "f"(a.y), "f"(a.z), "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
               : "memory");
}

// one 32-byte load through the read-only path (sm_100+ 256-bit vector load);
// p must be 32-byte aligned and not written during the kernel
__device__ __forceinline__ void ldg256(const float4 *p, float4 &a, float4 &b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

// Load pack fields: slots (d, v0, v1, [v2,] p, e, a) in the AoS order
//   2D: f4[0] = (d, vx, vy, p)  f4[1] = (e, a, 0, 0)
//   3D: f4[0] = (d, vx, vy, vz) f4[1] = (p, e, a, 0)
template <int D>
__device__ __forceinline__ prim<float, D> load_pack(const float4 *pk, int c) {
  float4 a, b;
  ldg256(pk + 2 * (size_t)c, a, b);
  prim<float, D> w;
  w.d = a.x;
  w.v[0] = a.y;
  w.v[1] = a.z;
  if (D == 2) {
    w.p = a.w;
    w.e = b.x;
    w.a = b.y;
  } else {
    w.v[D - 1] = a.w;
    w.p = b.x;
    w.e = b.y;
    w.a = b.z;
  }
  return w;
}

template <int D>
__device__ __forceinline__ void store_pack(float4 *pk, int c, float d, const float *v, float p,
                                           float e, float a) {
  if (D == 2) {
    pk[2 * (size_t)c] = make_float4(d, v[0], v[1], p);
    pk[2 * (size_t)c + 1] = make_float4(e, a, 0.f, 0.f);
  } else {
    pk[2 * (size_t)c] = make_float4(d, v[0], v[1], v[D - 1]);
    pk[2 * (size_t)c + 1] = make_float4(p, e, a, 0.f);
  }
}

// gradient record: g[k*D + i] = d u_k / d x_i, u = (d, v.., e, p, a)
template <int D>
__device__ __forceinline__ void load_grads(const float4 *gr, int c, float *g) {
  constexpr int G4 = layout<D>::GRAD4;
  float4 t[G4];
  if (G4 % 2 == 0) {  // 32-byte aligned records: 256-bit loads
#pragma unroll
    for (int q = 0; q < G4; q += 2) ldg256(gr + (size_t)G4 * c + q, t[q], t[q + 1]);
  } else {
#pragma unroll
    for (int q = 0; q < G4; ++q) t[q] = gr[(size_t)G4 * c + q];
  }
#pragma unroll
  for (int q = 0; q < G4; ++q) {
    g[4 * q] = t[q].x;
    g[4 * q + 1] = t[q].y;
    g[4 * q + 2] = t[q].z;
    g[4 * q + 3] = t[q].w;
  }
}

template <int D>
__device__ __forceinline__ void load_cen(const float4 *cc, int c, float *hi, float *lo) {
  if (D == 2) {
    const float4 t = cc[c];
    hi[0] = t.x; hi[1] = t.y; lo[0] = t.z; lo[1] = t.w;
  } else {
    float4 a, b;
    ldg256(cc + 2 * (size_t)c, a, b);  // hi and lo float4 in one 32-byte record
    hi[0] = a.x; hi[1] = a.y; hi[D - 1] = a.z;
    lo[0] = b.x; lo[1] = b.y; lo[D - 1] = b.z;
  }
}

__device__ __forceinline__ float2 split(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

// FP32 <-> FP64 conversions done with integer instructions, so they do not
// occupy the (narrow) FP64 pipe.  Values in the FP32 subnormal range flush to
// a signed zero; infinities and NaNs keep their class.
__device__ __forceinline__ double f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned sign = u & 0x80000000u;
  const unsigned ed = e == 0xffu ? 0x7ffu : e + 896u;
  const unsigned hi = e == 0 ? sign : (sign | (ed << 20) | ((u & 0x7fffffu) >> 3));
  const unsigned lo = e == 0 ? 0u : (u << 29);
  return __hiloint2double((int)hi, (int)lo);
}

// round to nearest even
__device__ __forceinline__ float d2f(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 896;  // FP32 biased exponent
  unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned r = lo & 0x1fffffffu;
  const unsigned up = (r > 0x10000000u) | ((r == 0x10000000u) & (m & 1u));
  unsigned f = (((unsigned)e) << 23) + m + up;  // a carry out of m bumps the exponent
  const bool nan = (hi & 0x7fffffffu) > 0x7ff00000u || ((hi & 0x7fffffffu) == 0x7ff00000u && lo);
  f = e <= 0 ? 0u : (e >= 255 ? (nan ? 0x7fc00000u : 0x7f800000u) : f);
  return __uint_as_float(sign | f);
}

// error-free sum s + x -> (s', err) (Knuth's two-sum).  The _rn intrinsics
// are never contracted into FMAs, which would break the identity.
__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
  hi = s;
  lo = __fadd_rn(lo, err);
}

// Double-float arithmetic: a value is the unevaluated sum hi + lo of two FP32
// numbers (about 48 significant bits).  Built from Knuth's two-sum, Dekker's
// fast two-sum and the FMA two-product; every operation is an explicit
// round-to-nearest intrinsic so the compiler neither contracts nor
// reassociates them.  It runs on the FP32 pipe, 64x wider than the FP64 pipe.
struct df {
  float hi, lo;
};
__device__ __forceinline__ df df_fast2(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_add(df x, df y) {
  const float s = __fadd_rn(x.hi, y.hi);
  const float bb = __fsub_rn(s, x.hi);
  const float err = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, bb)), __fsub_rn(y.hi, bb));
  return df_fast2(s, __fadd_rn(err, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, {-y.hi, -y.lo}); }
__device__ __forceinline__ df df_mul(df x, df y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  return df_fast2(p, e);
}
__device__ __forceinline__ df df_half(df x) { return {0.5f * x.hi, 0.5f * x.lo}; }
// x / y given r = RN(1/y.hi): quotient estimate, its double-float residual and
// one correction term
__device__ __forceinline__ df df_div(df x, df y, float r) {
  const float q1 = __fmul_rn(x.hi, r);
  const df res = df_sub(x, df_mul(y, {q1, 0.f}));
  return df_fast2(q1, __fmul_rn(res.hi, r));
}
// FP64 -> double-float (hi, lo) with hi + lo = x to about 2^-48 relative.
//
// The split needs no FP64 arithmetic.  hi = RN32(x) as in d2f; with
// x = M 2^(E-1075) (53-bit integer M, biased exponent E), x - hi is exactly
// n 2^(E-1075) for the signed 29-bit remainder n = (M mod 2^29) - 2^29 [hi
// rounded up], so lo = RN32(x - hi) is one integer-to-float conversion of n
// (I2F: on GB300 it issues to the FP64 pipe like F2F, but one of them costs
// less than an exact integer-only conversion in these ALU-bound kernels)
// times a power of two written into an exponent field.  |x| below 2^-74 gets
// lo = 0 (and hi = 0 below 2^-126, as in d2f).
__device__ __forceinline__ df df_from(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u;
  const int E = (int)((hi >> 20) & 0x7ffu);
  const int e = E - 896;
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned r = lo & 0x1fffffffu;
  const unsigned up = (r > 0x10000000u) | ((r == 0x10000000u) & (m & 1u));
  unsigned f = (((unsigned)e) << 23) + m + up;
  const bool nan = (hi & 0x7fffffffu) > 0x7ff00000u || ((hi & 0x7fffffffu) == 0x7ff00000u && lo);
  f = e <= 0 ? 0u : (e >= 255 ? (nan ? 0x7fc00000u : 0x7f800000u) : f);
  const int n = (int)r - (int)(up << 29);
  const int se = E - 948;  // FP32 biased exponent of 2^(E-1075)
  const float scale = (se >= 1 && se <= 254) ? __uint_as_float((unsigned)se << 23) : 0.f;
  const float l = __fmul_rn(__int2float_rn(n), scale);
  return {__uint_as_float(sign | f), __uint_as_float(__float_as_uint(l) ^ sign)};
}
// x + d in FP64 (two FP64 additions; x keeps all of its bits)
__device__ __forceinline__ double add_df(double x, df d) { return (x + f2d(d.hi)) + f2d(d.lo); }

// ---------------------------------------------------------------------------
// setup: FP32 geometry derived once from the FP64 mesh
// ---------------------------------------------------------------------------
template <int D>
__global__ void setup_cells(const fvh_mesh_view m, workspace w) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.num_cells) return;
  float hi[3], lo[3];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    const float2 s = split(m.cell_centroid[i][c]);
    hi[i] = s.x;
    lo[i] = s.y;
  }
  if (D == 2) {
    w.ccen[c] = make_float4(hi[0], hi[1], lo[0], lo[1]);
  } else {
    w.ccen[2 * (size_t)c] = make_float4(hi[0], hi[1], hi[D - 1], 0.f);
    w.ccen[2 * (size_t)c + 1] = make_float4(lo[0], lo[1], lo[D - 1], 0.f);
  }
  const float2 iv = split(1.0 / m.cell_volume[c]);
  w.inv_vol32[c] = iv.x;
  w.inv_vol_lo[c] = iv.y;
}

template <int D>
__global__ void setup_vertices(const fvh_mesh_view m, workspace w) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m.num_vertices) return;
  float hi[3], lo[3];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    const float2 s = split(m.vertex_coord[i][v]);
    hi[i] = s.x;
    lo[i] = s.y;
  }
  if (D == 2) {
    w.vcoord[v] = make_float4(hi[0], hi[1], lo[0], lo[1]);
  } else {
    w.vcoord[2 * (size_t)v] = make_float4(hi[0], hi[1], hi[D - 1], 0.f);
    w.vcoord[2 * (size_t)v + 1] = make_float4(lo[0], lo[1], lo[D - 1], 0.f);
  }
}

template <int D>
__global__ void setup_faces(const fvh_mesh_view m, workspace w) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.num_faces) return;
  const int c0 = m.face_cells[2 * (size_t)f], c1 = m.face_cells[2 * (size_t)f + 1];
  float n[3], d0[3], d1[3];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    n[i] = (float)m.face_normal[i][f];
    const double xf = m.face_centroid[i][f];
    d0[i] = (float)(xf - m.cell_centroid[i][c0]);
    d1[i] = c1 >= 0 ? (float)(xf - m.cell_centroid[i][c1]) : 0.f;
  }
  const float area = (float)m.face_area[f];
  if (D == 2) {
    w.fgeo[f] = make_float4(n[0], n[1], area, 0.f);
    w.fdx[f] = make_float4(d0[0], d0[1], d1[0], d1[1]);
  } else {
    w.fgeo[f] = make_float4(n[0], n[1], n[D - 1], area);
    w.fdx[2 * (size_t)f] = make_float4(d0[0], d0[1], d0[D - 1], 0.f);
    w.fdx[2 * (size_t)f + 1] = make_float4(d1[0], d1[1], d1[D - 1], 0.f);
  }
}

template <int D>
__device__ __forceinline__ void face_geo(const workspace &w, int f, float *n, float &area) {
  const float4 g = w.fgeo[f];
  n[0] = g.x;
  n[1] = g.y;
  if (D == 2) {
    area = g.z;
  } else {
    n[D - 1] = g.z;
    area = g.w;
  }
}

// block-wide FP32 maximum (valid in thread 0); all threads must call it
__device__ __forceinline__ float block_max_f(float v) {
  __shared__ float warp_max[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warp_max[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < (int)((blockDim.x + 31) >> 5) ? warp_max[lane] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}

// ---------------------------------------------------------------------------
// pack + dt partial maxima
// ---------------------------------------------------------------------------
// max over the faces of c of (a + |v.n|) A/V in FP32 (tasks.h:349-360)
template <int D>
__device__ __forceinline__ float cell_cfl(const fvh_mesh_view &m, const workspace &w, int c,
                                          const float *v, float a) {
  const float iv = w.inv_vol32[c];
  float r = 0.f;
  const int q0 = m.cell_face_offsets[c], nq = m.cell_face_offsets[c + 1] - q0;
  for (int k = 0; k < nq; ++k) {
    int f = m.cell_faces[q0 + k];
    f = f < 0 ? ~f : f;
    float n[D], area;
    face_geo<D>(w, f, n, area);
    r = smax((a + fabsf(phys::dot<float, D>(v, n))) * (area * iv), r);
  }
  return r;
}

// dt = min(CFL / max, t_f - t) from the maximum, in FP64 (tasks.h:362-375)
__device__ __forceinline__ void finish_dt(double dt_inv, double cfl, double final_time,
                                          const double *soln_time, double *dt_out,
                                          fvh_device_status *status) {
  const double max_dt = final_time - soln_time[0];
  if (dt_inv <= 0) {
    atomicMin(status, status_key(0, FVH_ERR_INFINITE_DT));
    dt_out[0] = 0;
  } else {
    double time_step = 1 / dt_inv;
    time_step *= cfl;
    dt_out[0] = smin(time_step, max_dt);
  }
}
// Also computes dt: every block publishes its maximum and the last block to
// finish (a ticket counter, reset by that block) reduces them in FP64.
template <int D>
__global__ void __launch_bounds__(kDtThreads)
pack_dt_kernel(const fvh_mesh_view m, const fvh_state_view s, workspace w, double *partial,
               const fvh_params p, const double *soln_time, double *dt_out,
               fvh_device_status *status, int rev, const fvh_state_view src, int copy) {
  // writes w.pack, the input of the predictor; with copy, the state is read
  // from src (host memory) and stored into s on the way (T is not an input)
  float dt_inv = 0.f;
  const fvh_state_view &in = copy ? src : s;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m.num_cells;
       i += gridDim.x * blockDim.x) {
    const int c = rev ? m.num_cells - 1 - i : i;
    double vd[D];
#pragma unroll
    for (int i = 0; i < D; ++i) vd[i] = in.velocity[i][c];
    const double dd = in.density[c], ed = in.internal_energy[c], pd = in.pressure[c],
                 ad = in.sound_speed[c];
    if (copy) {
      s.density[c] = dd;
#pragma unroll
      for (int i = 0; i < D; ++i) s.velocity[i][c] = vd[i];
      s.internal_energy[c] = ed;
      s.pressure[c] = pd;
      s.sound_speed[c] = ad;
    }
    float v[D];
#pragma unroll
    for (int i = 0; i < D; ++i) v[i] = d2f(vd[i]);
    const float a = d2f(ad);
    store_pack<D>(w.pack, c, d2f(dd), v, d2f(pd), d2f(ed), a);
    dt_inv = smax(cell_cfl<D>(m, w, c, v, a), dt_inv);
  }
  dt_inv = block_max_f(dt_inv);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = f2d(dt_inv);
    __threadfence();
    last = atomicAdd(w.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = 0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
    v = smax(reinterpret_cast<volatile const double *>(partial)[i], v);
  v = block_max(v);
  if (threadIdx.x == 0) {
    *w.ticket = 0u;
    finish_dt(v, p.cfl, p.final_time, soln_time, dt_out, status);
  }
}


// Batch form: per-problem maxima.  A block (or warp) whose cells all belong to
// one problem reduces first and issues one integer atomicMax on the FP32 bits
// (non-negative floats order like their bit patterns), so the result does not
// depend on the order of the atomics.
template <int D>
__global__ void __launch_bounds__(kDtThreads)
pack_dt_batch_kernel(const fvh_mesh_view m, const fvh_state_view s, workspace w,
                     const problem_map pm, int rev) {
  __shared__ int block_pr[kDtThreads / 32];
  __shared__ float block_v[kDtThreads / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = rev ? m.num_cells - 1 - i : i;
  float dti_c = 0.f;
  int pr = -1;
  if (i < m.num_cells) {
    pr = pm.cell_problem[c];
    float v[D];
#pragma unroll
    for (int i = 0; i < D; ++i) v[i] = d2f(s.velocity[i][c]);
    const float a = d2f(s.sound_speed[c]);
    store_pack<D>(w.pack, c, d2f(s.density[c]), v, d2f(s.pressure[c]),
                  d2f(s.internal_energy[c]), a);
    const float iv = w.inv_vol32[c];
    const int q0 = m.cell_face_offsets[c], nq = m.cell_face_offsets[c + 1] - q0;
    for (int k = 0; k < nq; ++k) {
      int f = m.cell_faces[q0 + k];
      f = f < 0 ? ~f : f;
      float n[D], area;
      face_geo<D>(w, f, n, area);
      dti_c = smax((a + fabsf(phys::dot<float, D>(v, n))) * (area * iv), dti_c);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int pr0 = __shfl_sync(0xffffffffu, pr, 0);
  const bool warp_uniform = __all_sync(0xffffffffu, pr == pr0);
  float wm = dti_c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) wm = fmaxf(wm, __shfl_xor_sync(0xffffffffu, wm, o));
  if (lane == 0) {
    block_pr[warp] = warp_uniform ? pr0 : -2;
    block_v[warp] = wm;
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
  bool block_uniform = true;
  for (int k = 0; k < nw; ++k) block_uniform = block_uniform && block_pr[k] == block_pr[0];
  if (block_uniform) {
    if (threadIdx.x == 0 && block_pr[0] >= 0) {
      float bm = 0.f;
      for (int k = 0; k < nw; ++k) bm = fmaxf(bm, block_v[k]);
      atomicMax(&pm.dtinv_bits[block_pr[0]], __float_as_uint(bm));
    }
  } else if (warp_uniform) {
    if (lane == 0 && pr0 >= 0) atomicMax(&pm.dtinv_bits[pr0], __float_as_uint(wm));
  } else if (pr >= 0) {
    atomicMax(&pm.dtinv_bits[pr], __float_as_uint(dti_c));
  }
}

// dt per problem; resets the accumulator for the next step.  A problem that
// has reached its final time gets dt = 0 and no longer changes.
__global__ void dt_final_batch_kernel(const problem_map pm, fvh_device_status dummy) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= pm.nproblems) return;
  const double dt_inv = f2d(__uint_as_float(pm.dtinv_bits[k]));
  pm.dtinv_bits[k] = 0u;
  const double max_dt = pm.final_time[k] - pm.t[k];
  if (pm.t[k] >= pm.final_time[k] - 1e-12 * fabs(pm.final_time[k])) {
    pm.dt[k] = 0;  // finished (the last clamped step can land an ulp short)
  } else if (dt_inv <= 0) {
    atomicMin(&pm.status[k], status_key(0, FVH_ERR_INFINITE_DT));
    pm.dt[k] = 0;
  } else {
    double time_step = 1 / dt_inv;
    time_step *= pm.cfl[k];
    time_step = smin(time_step, max_dt);
    pm.dt[k] = time_step > 0 ? time_step : 0.0;
  }
  (void)dummy;
}

// ---------------------------------------------------------------------------
// FP32 gradients + Barth-Jespersen vertex limiter
// ---------------------------------------------------------------------------
// Gradient and limiter arithmetic of one cell c0 (3D), one value at a time;
// nbr(k, u1, yh, yl) supplies neighbour k's pack values and centroid.
template <int D>
__device__ __forceinline__ void pack_values(const prim<float, D> &p, float *u) {
  int k = 0;
  u[k++] = p.d;
#pragma unroll
  for (int d = 0; d < D; ++d) u[k++] = p.v[d];
  u[k++] = p.e;
  u[k++] = p.p;
  u[k++] = p.a;
}

template <int D, bool LIMIT, int UNROLL, class NBR>
__device__ __forceinline__ void cell_gradients(const fvh_mesh_view &m, const workspace &w,
                                               int c0, const float *u0, const float *xh,
                                               const float *xl, int nn, NBR nbr) {
  constexpr int NV = D + 4;
  constexpr float tol = 1.e-9f;
  float M[6] = {0, 0, 0, 0, 0, 0};
  float b[NV][D];
  // neighbour extrema (tasks.h:232-236), taken in the same pass
  float umin[NV], umax[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) umin[k] = umax[k] = u0[k];
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int j = 0; j < D; ++j) b[k][j] = 0.f;
#pragma unroll UNROLL
  for (int q = 0; q < nn; ++q) {
    float u1[NV], yh[3], yl[3], dx[3];
    nbr(q, u1, yh, yl);
#pragma unroll
    for (int i = 0; i < D; ++i) dx[i] = (yh[i] - xh[i]) + (yl[i] - xl[i]);
    if (D == 2) {
      M[0] += dx[0] * dx[0];
      M[1] += dx[0] * dx[1];
      M[2] += dx[1] * dx[1];
    } else {
      M[0] += dx[0] * dx[0];
      M[1] += dx[0] * dx[1];
      M[2] += dx[0] * dx[D - 1];
      M[3] += dx[1] * dx[1];
      M[4] += dx[1] * dx[D - 1];
      M[5] += dx[D - 1] * dx[D - 1];
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const float du = u1[k] - u0[k];
#pragma unroll
      for (int j = 0; j < D; ++j) b[k][j] += du * dx[j];
      umin[k] = fminf(u1[k], umin[k]);
      umax[k] = fmaxf(u1[k], umax[k]);
    }
  }
  float g[NV][D];
  if (D == 2) {
    const float det = M[0] * M[2] - M[1] * M[1];
    const float inv = 1.f / det;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      g[k][0] = (b[k][0] * M[2] - b[k][1] * M[1]) * inv;
      g[k][1] = (b[k][1] * M[0] - b[k][0] * M[1]) * inv;
    }
  } else {
    const float a00 = M[0], a01 = M[1], a02 = M[2], a11 = M[3], a12 = M[4], a22 = M[5];
    const float c00 = a11 * a22 - a12 * a12;
    const float c01 = a02 * a12 - a01 * a22;
    const float c02 = a01 * a12 - a02 * a11;
    const float c11 = a00 * a22 - a02 * a02;
    const float c12 = a01 * a02 - a00 * a12;
    const float c22 = a00 * a11 - a01 * a01;
    const float inv = 1.f / (a00 * c00 + a01 * c01 + a02 * c02);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const float b0 = b[k][0], b1 = b[k][1], b2 = b[k][D - 1];
      g[k][0] = (c00 * b0 + c01 * b1 + c02 * b2) * inv;
      g[k][1] = (c01 * b0 + c11 * b1 + c12 * b2) * inv;
      g[k][D - 1] = (c02 * b0 + c12 * b1 + c22 * b2) * inv;
    }
  }
  if (LIMIT) {
    float dpos[NV], dneg[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) dpos[k] = dneg[k] = 0.f;
    const int r0 = m.cell_vertex_offsets[c0], nr = m.cell_vertex_offsets[c0 + 1] - r0;
    auto vertex = [&](const float *dxv) {
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        float du = 0.f;
#pragma unroll
        for (int i = 0; i < D; ++i) du += dxv[i] * g[k][i];
        dpos[k] = fmaxf(du, dpos[k]);
        dneg[k] = fminf(du, dneg[k]);
      }
    };
    for (int r = 0; r < nr; ++r) {
      float vh[3], vl[3], dxv[3];
      load_cen<D>(w.vcoord, m.cell_vertices[r0 + r], vh, vl);
#pragma unroll
      for (int i = 0; i < D; ++i) dxv[i] = __fadd_rn(__fsub_rn(vh[i], xh[i]), __fsub_rn(vl[i], xl[i]));
      vertex(dxv);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      float phi = 1.f;
      if (dpos[k] > tol) phi = fminf(phi, __fdividef(umax[k] - u0[k], dpos[k]));
      if (dneg[k] < -tol) phi = fminf(phi, __fdividef(umin[k] - u0[k], dneg[k]));
      phi = fmaxf(phi, 0.f);
#pragma unroll
      for (int i = 0; i < D; ++i) g[k][i] *= phi;
    }
  }
  constexpr int G4 = layout<D>::GRAD4;
  float flat[4 * G4];
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int i = 0; i < D; ++i) flat[k * D + i] = g[k][i];
#pragma unroll
  for (int q = NV * D; q < 4 * G4; ++q) flat[q] = 0.f;
#pragma unroll
  for (int q = 0; q < G4; ++q)
    w.grads[(size_t)G4 * c0 + q] =
        make_float4(flat[4 * q], flat[4 * q + 1], flat[4 * q + 2], flat[4 * q + 3]);
}

// Packed FP32 pairs (the FADD2/FMUL2/FFMA2 instructions of sm_100+): each lane
// rounds exactly like the scalar instruction.
__device__ __forceinline__ float2 bcast(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// The same arithmetic with packed pairs (2D).  The values stay in the pack's
// slot order (2D d vx vy p e a; 3D d vx vy vz p e a) so that adjacent slots
// form the FP32 pairs of one packed instruction:
// the differences, the least-squares sums, the solve, the vertex differences
// and the limiting take 3 pair instructions per dimension (plus one scalar in
// 3D) instead of 6 or 7 scalar ones.  u0 / the neighbours' records come as the
// two float4 of a pack; nbr(q, a, b, yh, yl) supplies neighbour q's record and
// centroid.  2D gradients 56.4 -> 54.6 us at 1024^2; in 3D the pairs keep more
// registers live in a kernel already at 96 and measured 3.6 % slower per step,
// so 3D takes the scalar form above.
template <int D, bool LIMIT, int UNROLL, class NBR, class VTX>
__device__ __forceinline__ void cell_gradients_pairs(const workspace &w, int c0, float4 a0,
                                                     float4 b0, const float *xh, const float *xl,
                                                     int nn, NBR nbr, int nr, VTX vtx) {
  constexpr int NV = D + 4;       // values (slots 0 .. NV-1 of the pack)
  constexpr int NP = NV / 2;      // slot pairs; 3D has slot NV-1 (a) left over
  constexpr bool ODD = NV % 2 == 1;
  constexpr float tol = 1.e-9f;
  // -u0 by slot (u_q - u0 = u_q + (-u0) exactly)
  const float nu0s[8] = {-a0.x, -a0.y, -a0.z, -a0.w, -b0.x, -b0.y, -b0.z, -b0.w};
  float2 nu0[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) nu0[p] = make_float2(nu0s[2 * p], nu0s[2 * p + 1]);
  const float2 nxh = make_float2(-xh[0], -xh[1]), nxl = make_float2(-xl[0], -xl[1]);
  // M = sum dx dx^T: 2D (m00, m01) m11; 3D (m00, m01) (m02, m12) m11 m22
  float2 mA = make_float2(0.f, 0.f), mB = make_float2(0.f, 0.f);
  float m11 = 0.f, m22 = 0.f;
  float2 bs[NP][D];  // sum (u_q - u0) dx_q for slot pairs
  float bo[D];       // and for the odd slot
  // neighbour extrema (tasks.h:232-236), taken in the same pass
  float umin[NV], umax[NV];
  {
    const float u0[8] = {a0.x, a0.y, a0.z, a0.w, b0.x, b0.y, b0.z, b0.w};
#pragma unroll
    for (int k = 0; k < NV; ++k) umin[k] = umax[k] = u0[k];
  }
#pragma unroll
  for (int j = 0; j < D; ++j) {
    bo[j] = 0.f;
#pragma unroll
    for (int p = 0; p < NP; ++p) bs[p][j] = make_float2(0.f, 0.f);
  }
#pragma unroll UNROLL
  for (int q = 0; q < nn; ++q) {
    float4 a, b;
    float yh[3], yl[3];
    nbr(q, a, b, yh, yl);
    const float2 dx01 = add2(add2(make_float2(yh[0], yh[1]), nxh),
                             add2(make_float2(yl[0], yl[1]), nxl));
    float dx[3] = {dx01.x, dx01.y, 0.f};
    if (D == 3) dx[2] = (yh[2] - xh[2]) + (yl[2] - xl[2]);
    mA = fma2(bcast(dx[0]), dx01, mA);
    m11 += dx[1] * dx[1];
    if (D == 3) {
      mB = fma2(dx01, bcast(dx[2]), mB);
      m22 += dx[2] * dx[2];
    }
    const float2 pr[4] = {make_float2(a.x, a.y), make_float2(a.z, a.w), make_float2(b.x, b.y),
                          make_float2(b.z, b.w)};
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const float2 du = add2(pr[p], nu0[p]);
#pragma unroll
      for (int j = 0; j < D; ++j) bs[p][j] = fma2(du, bcast(dx[j]), bs[p][j]);
    }
    if (ODD) {
      const float u1[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
      const float du = u1[NV - 1] + nu0s[NV - 1];
#pragma unroll
      for (int j = 0; j < D; ++j) bo[j] += du * dx[j];
    }
    {
      const float u1[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        umin[k] = fminf(u1[k], umin[k]);
        umax[k] = fmaxf(u1[k], umax[k]);
      }
    }
  }
  // closed-form solve, g = M^-1 b, per slot pair (go: the odd slot)
  float2 g[NP][D];
  float go[D];
  if (D == 2) {
    const float m00 = mA.x, m01 = mA.y;
    const float inv = 1.f / (m00 * m11 - m01 * m01);
    const float2 i11 = bcast(m11 * inv), i00 = bcast(m00 * inv), n01 = bcast(-m01 * inv);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      g[p][0] = fma2(bs[p][0], i11, mul2(bs[p][1], n01));
      g[p][1] = fma2(bs[p][1], i00, mul2(bs[p][0], n01));
    }
    go[0] = go[D - 1] = 0.f;
  } else {
    const float a00 = mA.x, a01 = mA.y, a02 = mB.x, a12 = mB.y, a11 = m11, a22 = m22;
    const float c00 = a11 * a22 - a12 * a12;
    const float c01 = a02 * a12 - a01 * a22;
    const float c02 = a01 * a12 - a02 * a11;
    const float c11 = a00 * a22 - a02 * a02;
    const float c12 = a01 * a02 - a00 * a12;
    const float c22 = a00 * a11 - a01 * a01;
    const float inv = 1.f / (a00 * c00 + a01 * c01 + a02 * c02);
    const float2 k00 = bcast(c00 * inv), k01 = bcast(c01 * inv), k02 = bcast(c02 * inv),
                 k11 = bcast(c11 * inv), k12 = bcast(c12 * inv), k22 = bcast(c22 * inv);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const float2 x = bs[p][0], y = bs[p][1], z = bs[p][D - 1];
      g[p][0] = fma2(k00, x, fma2(k01, y, mul2(k02, z)));
      g[p][1] = fma2(k01, x, fma2(k11, y, mul2(k12, z)));
      g[p][D - 1] = fma2(k02, x, fma2(k12, y, mul2(k22, z)));
    }
    const float x = bo[0], y = bo[1], z = bo[D - 1];
    go[0] = k00.x * x + (k01.x * y + k02.x * z);
    go[1] = k01.x * x + (k11.x * y + k12.x * z);
    go[D - 1] = k02.x * x + (k12.x * y + k22.x * z);
  }
  if (LIMIT) {
    float dpos[NV], dneg[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) dpos[k] = dneg[k] = 0.f;
    for (int r = 0; r < nr; ++r) {
      float vh[3], vl[3], dxv[3];
      vtx(r, vh, vl);
#pragma unroll
      for (int i = 0; i < D; ++i) dxv[i] = __fadd_rn(__fsub_rn(vh[i], xh[i]), __fsub_rn(vl[i], xl[i]));
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        float2 du = mul2(g[p][0], bcast(dxv[0]));
#pragma unroll
        for (int i = 1; i < D; ++i) du = fma2(g[p][i], bcast(dxv[i]), du);
        dpos[2 * p] = fmaxf(du.x, dpos[2 * p]);
        dneg[2 * p] = fminf(du.x, dneg[2 * p]);
        dpos[2 * p + 1] = fmaxf(du.y, dpos[2 * p + 1]);
        dneg[2 * p + 1] = fminf(du.y, dneg[2 * p + 1]);
      }
      if (ODD) {
        float du = go[0] * dxv[0];
#pragma unroll
        for (int i = 1; i < D; ++i) du += go[i] * dxv[i];
        dpos[NV - 1] = fmaxf(du, dpos[NV - 1]);
        dneg[NV - 1] = fminf(du, dneg[NV - 1]);
      }
    }
    float phi[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      phi[k] = 1.f;
      if (dpos[k] > tol) phi[k] = fminf(phi[k], __fdividef(umax[k] + nu0s[k], dpos[k]));
      if (dneg[k] < -tol) phi[k] = fminf(phi[k], __fdividef(umin[k] + nu0s[k], dneg[k]));
      phi[k] = fmaxf(phi[k], 0.f);
    }
#pragma unroll
    for (int i = 0; i < D; ++i) {
#pragma unroll
      for (int p = 0; p < NP; ++p) g[p][i] = mul2(g[p][i], make_float2(phi[2 * p], phi[2 * p + 1]));
      if (ODD) go[i] *= phi[NV - 1];
    }
  }
  // gradient record in value order (d, v.., e, p, a): pack slots
  // 2D (0, 1, 2, 4, 3, 5), 3D (0, 1, 2, 3, 5, 4, 6)
  float gs[NV + 1][D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      gs[2 * p][i] = g[p][i].x;
      gs[2 * p + 1][i] = g[p][i].y;
    }
    gs[NV - 1 + (ODD ? 0 : 1)][i] = go[i];  // 2D: an unused row
  }
  constexpr int G4 = layout<D>::GRAD4;
  float flat[4 * G4];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const int sl = k < D + 1 ? k : (k == D + 1 ? D + 2 : (k == D + 2 ? D + 1 : D + 3));
#pragma unroll
    for (int i = 0; i < D; ++i) flat[k * D + i] = gs[sl][i];
  }
#pragma unroll
  for (int q = NV * D; q < 4 * G4; ++q) flat[q] = 0.f;
#pragma unroll
  for (int q = 0; q < G4; ++q)
    w.grads[(size_t)G4 * c0 + q] =
        make_float4(flat[4 * q], flat[4 * q + 1], flat[4 * q + 2], flat[4 * q + 3]);
}

// Neighbour records are loaded as the loop reaches them.  3D keeps
// 7 x 3 gradient sums, 14 extrema and the 3x3 system live: 96 registers
// there (5 blocks of 128 per SM; measured faster than 128 registers with 4
// blocks, or 80 with spills), 64 in 2D.
template <int D, bool LIMIT, int BS>
__global__ void __launch_bounds__(BS, (D == 2 ? 1024 : 640) / BS)
gradients_kernel(const fvh_mesh_view m, workspace w, const float4 *__restrict__ pk, int rev) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < m.num_cells; i += gridDim.x * BS) {
    const int c0 = rev ? m.num_cells - 1 - i : i;
    float xh[3], xl[3];
    load_cen<D>(w.ccen, c0, xh, xl);
    const int q0 = m.cell_nbr_offsets[c0], nn = m.cell_nbr_offsets[c0 + 1] - q0;
    if (D == 2) {
      float4 a0, b0;
      ldg256(pk + 2 * (size_t)c0, a0, b0);
      const int r0 = m.cell_vertex_offsets[c0], nr = m.cell_vertex_offsets[c0 + 1] - r0;
      cell_gradients_pairs<D, LIMIT, 4>(
          w, c0, a0, b0, xh, xl, nn,
          [&](int q, float4 &a, float4 &b, float *yh, float *yl) {
            const int c1 = m.cell_nbrs[q0 + q];
            ldg256(pk + 2 * (size_t)c1, a, b);
            load_cen<D>(w.ccen, c1, yh, yl);
          },
          nr, [&](int r, float *vh, float *vl) { load_cen<D>(w.vcoord, m.cell_vertices[r0 + r], vh, vl); });
    } else {
      float u0[D + 4];
      pack_values<D>(load_pack<D>(pk, c0), u0);
      cell_gradients<D, LIMIT, 4>(m, w, c0, u0, xh, xl, nn,
                                  [&](int q, float *u1, float *yh, float *yl) {
                                    const int c1 = m.cell_nbrs[q0 + q];
                                    pack_values<D>(load_pack<D>(pk, c1), u1);
                                    load_cen<D>(w.ccen, c1, yh, yl);
                                  });
    }
  }
}

// ---------------------------------------------------------------------------
// 2D gradients from records staged in shared memory by the bulk-copy (TMA)
// engine
// ---------------------------------------------------------------------------
// The gathers of gradients_kernel are dependent loads (offsets -> neighbour
// ids -> records) that keep it latency-bound.  Here the cells are taken in
// chunks of up to kStageCells cells that lie close together (consecutive in
// the Morton order of the cell centroids: a compact tile of a box), one cell
// per thread.  A chunk reads the pack and centroid of a set of cells (its own
// and their vertex neighbours) and the coordinates of its cells' vertices; on
// a mesh numbered row by row these sets are a few runs of consecutive ids.  The
// setup lists each chunk's runs and packs, per cell, its own record's position
// and those of its neighbours and vertices in the chunk's staged set (a byte
// each, four to a 32-bit word), and sizes the stage buffers for the mesh's
// largest chunk.  A persistent kernel posts the copies of chunk i+1 (one bulk
// copy per run and array, plus one for the chunk's topology; completion
// counted on an mbarrier) while its threads compute chunk i from shared memory
// with the arithmetic of gradients_kernel (cell_gradients_pairs), so both
// kernels give the same bits.
constexpr int kStageCells = 128;      // cells per chunk = threads per block
constexpr int kStageMaxCells = 256;   // staged cell records per chunk (byte slots)
constexpr int kStageMaxVerts = 256;   // staged vertex records per chunk
constexpr int kStageMaxBytes = 24576; // one stage buffer at most (two per block)
constexpr int kStageWaitPolls = 1 << 22;  // bounded waits on a chunk's copies

template <bool LIMIT>
__global__ void __launch_bounds__(kStageCells)
gradients_staged_kernel(const fvh_mesh_view m, workspace w, const float4 *__restrict__ pk,
                        stage_tables t, int rev, fvh_device_status *status) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar[2];
  const int tid = threadIdx.x;
  auto chunk_at = [&](int i) { return rev ? t.nchunks - 1 - i : i; };
  // posts the copies of chunk k into stage buffer b (warp 0)
  auto post = [&](int k, int b) {
    const int r0 = t.run_off[k], nr = t.run_off[k + 1] - r0;
    const long long tb0 = t.topo_off[k];
    const unsigned topo_bytes = (unsigned)(t.topo_off[k + 1] - tb0);
    unsigned char *base = smem + (size_t)b * t.stage_bytes;
    // this buffer's earlier reads (ordered by the block barrier) come before
    // the copies that overwrite it
    tma::fence_proxy_async_shared();
    if (tid == 0) {
      tma::mbar_arrive_expect_tx(&bar[b], t.bytes[k]);
      tma::bulk_g2s(base + t.topo_at, reinterpret_cast<const unsigned char *>(t.topo) + tb0,
                    topo_bytes, &bar[b]);
    }
    __syncwarp();
    for (int r = tid; r < nr; r += 32) {
      const stage_run run = t.runs[r0 + r];
      if (run.kind == 0) {
        tma::bulk_g2s(base + (size_t)run.slot * 32, pk + 2 * (size_t)run.first,
                      (unsigned)run.count * 32u, &bar[b]);
        tma::bulk_g2s(base + t.cen_at + (size_t)run.slot * 16, w.ccen + run.first,
                      (unsigned)run.count * 16u, &bar[b]);
      } else {
        tma::bulk_g2s(base + t.vtx_at + (size_t)run.slot * 16, w.vcoord + run.first,
                      (unsigned)run.count * 16u, &bar[b]);
      }
    }
  };
  if (tid == 0) {
    tma::mbar_init(&bar[0], 1);
    tma::mbar_init(&bar[1], 1);
    tma::fence_barrier_init();
  }
  __syncthreads();
  // copies posted into / phases consumed from each buffer (the same in every
  // thread: the decisions below are uniform across the block)
  int posted[2] = {0, 0}, used[2] = {0, 0};
  if ((int)blockIdx.x < t.nchunks) {
    if (tid < 32) post(chunk_at(blockIdx.x), 0);
    posted[0] = 1;
  }
  int it = 0;
  for (int i = blockIdx.x; i < t.nchunks; i += gridDim.x, ++it) {
    const int b = it & 1;
    // the other buffer was last read by the previous chunk, before the
    // barrier that ended it
    if (i + (int)gridDim.x < t.nchunks) {
      if (tid < 32) post(chunk_at(i + gridDim.x), b ^ 1);
      ++posted[b ^ 1];
    }
    const int k = chunk_at(i);
    const int c0 = t.cells[(size_t)k * kStageCells + tid];
    const bool landed = tma::mbar_wait_bounded(&bar[b], (unsigned)(used[b] & 1), kStageWaitPolls);
    ++used[b];
    const unsigned char *base = smem + (size_t)b * t.stage_bytes;
    const float4 *spk = reinterpret_cast<const float4 *>(base);
    const float4 *scen = reinterpret_cast<const float4 *>(base + t.cen_at);
    const float4 *svtx = reinterpret_cast<const float4 *>(base + t.vtx_at);
    const unsigned *topo = reinterpret_cast<const unsigned *>(base + t.topo_at);
    if (landed && c0 >= 0) {
      // the cell's record: word 0 = own slot | nn << 8 | nr << 16, then the
      // neighbour slots and the vertex slots, four bytes to a word each
      const unsigned *rec = topo + (reinterpret_cast<const unsigned short *>(topo)[tid]);
      const unsigned head = rec[0];
      const int own = head & 0xffu, nn = (head >> 8) & 0xffu, nr = (head >> 16) & 0xffu;
      const unsigned *nslot = rec + 1, *vslot = rec + 1 + ((nn + 3) >> 2);
      auto byte_at = [](const unsigned *wd, int i) { return (int)((wd[i >> 2] >> ((i & 3) * 8)) & 0xffu); };
      const float4 a0 = spk[2 * own], b0 = spk[2 * own + 1];
      const float4 x0 = scen[own];
      const float xh[3] = {x0.x, x0.y, 0.f}, xl[3] = {x0.z, x0.w, 0.f};
      cell_gradients_pairs<2, LIMIT, 4>(
          w, c0, a0, b0, xh, xl, nn,
          [&](int q, float4 &a, float4 &bb, float *yh, float *yl) {
            const int sl = byte_at(nslot, q);
            a = spk[2 * sl];
            bb = spk[2 * sl + 1];
            const float4 y = scen[sl];
            yh[0] = y.x; yh[1] = y.y; yl[0] = y.z; yl[1] = y.w;
          },
          nr,
          [&](int r, float *vh, float *vl) {
            const float4 v = svtx[byte_at(vslot, r)];
            vh[0] = v.x; vh[1] = v.y; vl[0] = v.z; vl[1] = v.w;
          });
    }
    // the one block barrier of a chunk: every thread is done with this
    // buffer before it is posted again, and a wait that ran out anywhere
    // stops the whole block
    if (__syncthreads_or(!landed)) {
      // report, then wait (bounded) for every posted copy before leaving, so
      // none lands in shared memory this block no longer owns
      if (tid == 0) atomicMin(status, status_key(t.cells[(size_t)k * kStageCells], FVH_ERR_TIMEOUT));
      for (int bb = 0; bb < 2; ++bb)  // (a phase that completed returns at once)
        if (posted[bb] > 0)
          tma::mbar_wait_bounded(&bar[bb], (unsigned)((posted[bb] - 1) & 1), kStageWaitPolls);
      return;
    }
  }
}

// ---------------------------------------------------------------------------
// cell-centric flux + FP64 update
// ---------------------------------------------------------------------------
// reconstruct the state of cell c at offset dx (x_f - x_c) from pack + grads
template <int D, bool SECOND>
__device__ __forceinline__ prim<float, D> recon(const workspace &w, const float4 *pk, int c,
                                                const float *dx, bool swap);

// reconstruction of cell values u (pack) with gradients g at offset dx
template <int D, bool SECOND>
__device__ __forceinline__ prim<float, D> recon_from(prim<float, D> u, const float *g,
                                                     const float *dx, bool swap) {
  if (SECOND) {
    // gradient rows: 0 d, 1..D v, D+1 e, D+2 p, D+3 a
    const int ge = swap ? D + 2 : D + 1;  // row added to the energy slot
    const int gp = swap ? D + 1 : D + 2;  // row added to the pressure slot
#pragma unroll
    for (int i = 0; i < D; ++i) {
      u.d += dx[i] * g[0 * D + i];
#pragma unroll
      for (int d = 0; d < D; ++d) u.v[d] += dx[i] * g[(1 + d) * D + i];
      u.p += dx[i] * g[gp * D + i];
      u.e += dx[i] * g[ge * D + i];
      u.a += dx[i] * g[(D + 3) * D + i];
    }
  }
  return u;
}

template <int D, bool SECOND>
__device__ __forceinline__ prim<float, D> recon(const workspace &w, const float4 *pk, int c,
                                                const float *dx, bool swap) {
  float g[4 * layout<D>::GRAD4];
  if (SECOND) load_grads<D>(w.grads, c, g);
  return recon_from<D, SECOND>(load_pack<D>(pk, c), g, dx, swap);
}

// Area-scaled flux of face f in its own orientation (cells(f)[0] -> [1]),
// F[k] = RN(flux_k * A_f).  Both cells of a face and the face kernel get the
// same bits from it.
template <int D, int KIND, bool SECOND>
__device__ __forceinline__ void face_flux_area(const fvh_mesh_view &m, const workspace &w,
                                               const float4 *__restrict__ pk, int f, int swap,
                                               int outflow, float *F) {
  const int2 cc = reinterpret_cast<const int2 *>(m.face_cells)[f];
  float n[D], area;
  face_geo<D>(w, f, n, area);
  float dx0[D], dx1[D];
  if (D == 2) {
    const float4 t = w.fdx[f];
    dx0[0] = t.x; dx0[1] = t.y; dx1[0] = t.z; dx1[1] = t.w;
  } else {
    const float4 a = w.fdx[2 * (size_t)f], b = w.fdx[2 * (size_t)f + 1];
    dx0[0] = a.x; dx0[1] = a.y; dx0[D - 1] = a.z;
    dx1[0] = b.x; dx1[1] = b.y; dx1[D - 1] = b.z;
  }
  const prim<float, D> wl = recon<D, SECOND>(w, pk, cc.x, dx0, swap != 0);
  if (cc.y >= 0) {
    const prim<float, D> wr = recon<D, SECOND>(w, pk, cc.y, dx1, swap != 0);
    phys::riemann<float, D, KIND>(wl, wr, n, F);
  } else if (outflow) {
    phys::phys_flux<float, D>(wl, n, F);
  } else {
    phys::wall<float, D>(wl, n, F);
  }
#pragma unroll
  for (int k = 0; k < D + 2; ++k) F[k] = __fmul_rn(F[k], area);
}

// Constants of the conservative update.
struct update_consts {
  df gm1;        // gamma - 1
  float ggm1;    // gamma (gamma - 1), for the FP32 sound speed
  float factor;  // fraction of dt this stage advances (0.5)
  double inv_cv; // 1 / cv
  int unit_cv;   // cv == 1: T = e exactly
};

// x < 0 (not -0, not +NaN) from the bits, off the FP64 pipe
__device__ __forceinline__ bool negative(double x) {
  return (unsigned long long)__double_as_longlong(x) > 0x8000000000000000ull;
}

// Conservative update of cell c from its compensated face sums
// (update_state_from_flux + update_state_from_energy, tasks.h:589-659), in
// the increment form
//   rho' = rho + dU0,   v' = v + (dUm - v dU0) / rho',
//   e'   = e + (dUE - (e + |v|^2/2) dU0) / rho' - v.dv - |dv|^2/2
// with dU = (face sum) dt / V and all increments in double-float, so
// rho'(e' + |v'|^2/2) is the old total energy plus dUE to about 2^-48 relative.
//
// STAGE 0 (predictor) writes no FP64 state: it keeps its increments (d rho,
// d v.., d e) in w.delta and writes the FP32 pack of the predicted state.
// STAGE 1 (corrector) rebuilds the predicted state from the FP64 state and
// those increments, adds its own, and writes the FP64 state as
//   x_new = x + (d_predictor + d_corrector)
// so every FP64 value takes one double-float increment per time step and
// keeps all of its bits.  FP64 pipe per step: 2D+5 additions (the splits run
// on the integer pipe).
//
// pk_out: the predictor's output pack; for the corrector (when not null) the
// pack of the next step, equal to what pack_dt writes from the new FP64 state,
// with the FP32 velocity and sound speed also returned in vnext / anext.
template <int D, int STAGE>
__device__ __forceinline__ void cell_update(const fvh_state_view &s, const workspace &w,
                                            float4 *__restrict__ pk_out, const problem_map &pm,
                                            int c, int pr, df dts, const float *shi,
                                            const float *slo, const update_consts &k,
                                            float *vnext = nullptr, float *anext = nullptr,
                                            const fvh_state_view *out = nullptr) {
  constexpr int L4 = layout<D>::DEL4;
  const df scale = df_mul(dts, {w.inv_vol32[c], w.inv_vol_lo[c]});
  df du[D + 2];
#pragma unroll
  for (int q = 0; q < D + 2; ++q) du[q] = df_mul({shi[q], slo[q]}, scale);
  const double den0 = s.density[c], e0 = s.internal_energy[c];
  double vel[D];
  df rho = df_from(den0), e = df_from(e0), v[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    vel[i] = s.velocity[i][c];
    v[i] = df_from(vel[i]);
  }
  float pv[4 * L4];  // predictor increments: (d rho, d v.., d e) as (hi, lo) pairs
  if (STAGE == 1) {
    const float4 *dp = w.delta + (size_t)L4 * c;
    float4 t[L4];
    if (L4 == 2) {
      ldg256(dp, t[0], t[1]);
    } else {
#pragma unroll
      for (int q = 0; q < L4; ++q) t[q] = dp[q];
    }
#pragma unroll
    for (int q = 0; q < L4; ++q) {
      pv[4 * q] = t[q].x;
      pv[4 * q + 1] = t[q].y;
      pv[4 * q + 2] = t[q].z;
      pv[4 * q + 3] = t[q].w;
    }
    rho = df_add(rho, {pv[0], pv[1]});
#pragma unroll
    for (int i = 0; i < D; ++i) v[i] = df_add(v[i], {pv[2 + 2 * i], pv[3 + 2 * i]});
    e = df_add(e, {pv[2 * D + 2], pv[2 * D + 3]});
  }
  const df rho2 = df_add(rho, du[0]);
  const float r = __frcp_rn(rho2.hi);
  df k0 = {0.f, 0.f}, dv[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    k0 = df_add(k0, df_mul(v[i], v[i]));
    dv[i] = df_div(df_sub(du[1 + i], df_mul(v[i], du[0])), rho2, r);
  }
  df de = df_div(df_sub(du[D + 1], df_mul(df_add(e, df_half(k0)), du[0])), rho2, r);
  df vdv = {0.f, 0.f}, dv2 = {0.f, 0.f};
#pragma unroll
  for (int i = 0; i < D; ++i) {
    vdv = df_add(vdv, df_mul(v[i], dv[i]));
    dv2 = df_add(dv2, df_mul(dv[i], dv[i]));
  }
  de = df_sub(de, df_add(vdv, df_half(dv2)));
  const df e2 = df_add(e, de);
  const df pd = df_mul(k.gm1, df_mul(rho2, e2));
  const float a = sqrtf(k.ggm1 * e2.hi);
  if (STAGE == 0) {
    float t[4 * L4];
    t[0] = du[0].hi;
    t[1] = du[0].lo;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      t[2 + 2 * i] = dv[i].hi;
      t[3 + 2 * i] = dv[i].lo;
    }
    t[2 * D + 2] = de.hi;
    t[2 * D + 3] = de.lo;
#pragma unroll
    for (int q = 2 * D + 4; q < 4 * L4; ++q) t[q] = 0.f;
    float4 *dp = w.delta + (size_t)L4 * c;
    if (L4 == 2) {
      stg256(dp, make_float4(t[0], t[1], t[2], t[3]), make_float4(t[4], t[5], t[6], t[7]));
    } else {
#pragma unroll
      for (int q = 0; q < L4; ++q)
        dp[q] = make_float4(t[4 * q], t[4 * q + 1], t[4 * q + 2], t[4 * q + 3]);
    }
    float vf[D];
#pragma unroll
    for (int i = 0; i < D; ++i) vf[i] = df_add(v[i], dv[i]).hi;
    store_pack<D>(pk_out, c, rho2.hi, vf, pd.hi, e2.hi, a);
    if (e2.hi < 0.f || rho2.hi < 0.f)
      atomicMin(&pm.status[pr], status_key(c, FVH_ERR_NEGATIVE_STATE));
  } else {
    const double mass = add_df(den0, df_add({pv[0], pv[1]}, du[0]));
#pragma unroll
    for (int i = 0; i < D; ++i)
      vel[i] = add_df(vel[i], df_add({pv[2 + 2 * i], pv[3 + 2 * i]}, dv[i]));
    const double en = add_df(e0, df_add({pv[2 * D + 2], pv[2 * D + 3]}, de));
    const double p = f2d(pd.hi) + f2d(pd.lo);
    s.density[c] = mass;
#pragma unroll
    for (int i = 0; i < D; ++i) s.velocity[i][c] = vel[i];
    s.internal_energy[c] = en;
    s.pressure[c] = p;
    s.temperature[c] = k.unit_cv ? en : en * k.inv_cv;
    s.sound_speed[c] = f2d(a);
    if (out) {  // the caller's copy of the state (host memory)
      out->density[c] = mass;
#pragma unroll
      for (int i = 0; i < D; ++i) out->velocity[i][c] = vel[i];
      out->internal_energy[c] = en;
      out->pressure[c] = p;
      out->temperature[c] = k.unit_cv ? en : en * k.inv_cv;
      out->sound_speed[c] = f2d(a);
    }
    if (pk_out) {
#pragma unroll
      for (int i = 0; i < D; ++i) vnext[i] = d2f(vel[i]);
      *anext = a;
      store_pack<D>(pk_out, c, d2f(mass), vnext, d2f(p), d2f(en), a);
    }
    if (negative(en) || negative(mass))
      atomicMin(&pm.status[pr], status_key(c, FVH_ERR_NEGATIVE_STATE));
  }
}

constexpr int kCflMaxBlocks = 1216;

// The corrector's dt for the next step: the CFL maximum of the cells' new
// state, one integer atomicMax per block on the FP32 bits (order-independent),
// and the last block to finish computes dt as pack_dt would.
struct next_dt {
  double cfl = 0, final_time = 0;
  const double *soln_time = nullptr;
  double *dt = nullptr;
  fvh_device_status *status = nullptr;
  bool write_next = false;  // the corrector writes the next step's pack and dt
  fvh_state_view out{};     // with has_out, the corrector also writes the state here
  int has_out = 0;
  int batch = 0;            // per-problem maxima (problem_map::dtinv_bits) instead
};

// Batch form: the next step's per-problem CFL maxima.  Lanes that arrive
// together and share a problem combine their values; one integer atomicMax on
// the FP32 bits per group (order-independent, as in pack_dt_batch).
__device__ __forceinline__ void problem_cfl(const problem_map &pm, int pr, float v) {
  const unsigned active = __activemask();
  const unsigned grp = __match_any_sync(active, pr);
  const unsigned mx = __reduce_max_sync(grp, __float_as_uint(v));
  if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(&pm.dtinv_bits[pr], mx);
}

__device__ __forceinline__ void finish_cfl(const workspace &w, const next_dt &nd, float dt_inv) {
  dt_inv = block_max_f(dt_inv);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    atomicMax(w.dtinv_max, __float_as_uint(dt_inv));
    __threadfence();
    last = atomicAdd(w.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    const float mx = __uint_as_float(atomicExch(w.dtinv_max, 0u));
    *w.ticket = 0u;
    finish_dt(f2d(mx), nd.cfl, nd.final_time, nd.soln_time, nd.dt, nd.status);
  }
}

// CFL maximum of a cell the corrector leaves untouched (its problem is at its
// final time): from its current pack record.
template <int D>
__device__ __forceinline__ float untouched_cfl(const fvh_mesh_view &m, const workspace &w,
                                               int c) {
  const float4 a = w.pack[2 * (size_t)c], b = w.pack[2 * (size_t)c + 1];
  float v[D];
  v[0] = a.y;
  v[1] = a.z;
  if (D == 3) v[D - 1] = a.w;
  return cell_cfl<D>(m, w, c, v, D == 2 ? b.y : b.z);
}

// Per-thread cache of the stage's dt for the problem of the current cell; the
// problem's solution time is advanced by its first cell.  Returns false for a
// finished problem (dt == 0), whose state is left untouched.
struct stage_dt {
  int pr = -1;
  bool live = false;
  df dts;
  __device__ __forceinline__ bool at(const problem_map &pm, int c, int cpr, float factor) {
    if (cpr != pr) {
      pr = cpr;
      const double dt = pm.dt[pr];
      live = (__double_as_longlong(dt) << 1) != 0;
      dts = df_from(dt);
      dts.hi *= factor;  // factor is a power of two: exact
      dts.lo *= factor;
    }
    if (c == (pm.cell_problem ? pm.first_cell[pr] : 0))
      pm.t[pr] = pm.t[pr] + pm.dt[pr] * (double)factor;
    return live;
  }
};

// Cell-centric schedule: each cell evaluates the fluxes of its own faces.
// NEXT (corrector): 0 = nothing more, 2 = the next step's pack and dt, 3 = the
// next step's pack and per-problem CFL maxima (batch).
template <int D, int KIND, bool SECOND, int BS, int STAGE, int NEXT = 0>
__global__ void __launch_bounds__(BS, 1024 / BS)
flux_update_kernel(const fvh_mesh_view m, const fvh_state_view s, workspace w,
                   const float4 *__restrict__ pk_in, float4 *__restrict__ pk_out,
                   const problem_map pm, const update_consts uc, int swap, int outflow,
                   int rev, const next_dt nd, const fvh_state_view out, int has_out) {
  // Reads pk_in (all cells) and the cell's own FP64 state; the predictor writes
  // the cell's increments and pk_out record, the corrector its FP64 state.
  stage_dt sdt;
  float dt_inv = 0.f;
  for (int i = blockIdx.x * BS + threadIdx.x; i < m.num_cells; i += gridDim.x * BS) {
    const int c = rev ? m.num_cells - 1 - i : i;
    const int pr = pm.cell_problem ? pm.cell_problem[c] : 0;
    if (!sdt.at(pm, c, pr, uc.factor)) {
      if (NEXT == 2) dt_inv = smax(untouched_cfl<D>(m, w, c), dt_inv);
      if (NEXT == 3) problem_cfl(pm, pr, untouched_cfl<D>(m, w, c));
      continue;
    }
    // face sums in FP32 with error-free two-sum compensation (hi + lo carries
    // about 48 bits)
    float shi[D + 2], slo[D + 2];
#pragma unroll
    for (int k = 0; k < D + 2; ++k) shi[k] = slo[k] = 0.f;
    const int q0 = m.cell_face_offsets[c], nq = m.cell_face_offsets[c + 1] - q0;
#pragma unroll 2
    for (int k = 0; k < nq; ++k) {
      const int sf = m.cell_faces[q0 + k];
      float F[D + 2];
      face_flux_area<D, KIND, SECOND>(m, w, pk_in, sf < 0 ? ~sf : sf, swap, outflow, F);
#pragma unroll
      for (int k = 0; k < D + 2; ++k) two_sum_acc(shi[k], slo[k], sf >= 0 ? -F[k] : F[k]);
    }
    float vn[D], an;
    cell_update<D, STAGE>(s, w, pk_out, pm, c, pr, sdt.dts, shi, slo, uc, vn, &an,
                          STAGE == 1 && has_out ? &out : nullptr);
    if (NEXT == 2) dt_inv = smax(cell_cfl<D>(m, w, c, vn, an), dt_inv);
    if (NEXT == 3) problem_cfl(pm, pr, cell_cfl<D>(m, w, c, vn, an));
  }
  if (NEXT == 2) finish_cfl(w, nd, dt_inv);
}

// Face schedule, part 1: one flux per face into the FP32 face-flux array.
template <int D, int KIND, bool SECOND, int BS>
__global__ void __launch_bounds__(BS, 1024 / BS)
face_flux_kernel(const fvh_mesh_view m, workspace w, const float4 *__restrict__ pk_in, int swap,
                 int outflow, int rev) {
  constexpr int F4 = layout<D>::FLUX4;
  for (int i = blockIdx.x * BS + threadIdx.x; i < m.num_faces; i += gridDim.x * BS) {
    const int f = rev ? m.num_faces - 1 - i : i;
    float F[4 * F4];
    face_flux_area<D, KIND, SECOND>(m, w, pk_in, f, swap, outflow, F);
#pragma unroll
    for (int k = D + 2; k < 4 * F4; ++k) F[k] = 0.f;
#pragma unroll
    for (int q = 0; q < F4; ++q)
      w.fflux[(size_t)F4 * f + q] = make_float4(F[4 * q], F[4 * q + 1], F[4 * q + 2], F[4 * q + 3]);
  }
}

// Face schedule, part 2: cell-centric gather of the face-flux array + update.
template <int D, int BS, int STAGE, int NEXT = 0>
__global__ void __launch_bounds__(BS, 1024 / BS)
gather_update_kernel(const fvh_mesh_view m, const fvh_state_view s, workspace w,
                     float4 *__restrict__ pk_out, const problem_map pm,
                     const update_consts uc, int rev, const next_dt nd,
                     const fvh_state_view out, int has_out) {
  constexpr int F4 = layout<D>::FLUX4;
  stage_dt sdt;
  float dt_inv = 0.f;
  for (int i = blockIdx.x * BS + threadIdx.x; i < m.num_cells; i += gridDim.x * BS) {
    const int c = rev ? m.num_cells - 1 - i : i;
    const int pr = pm.cell_problem ? pm.cell_problem[c] : 0;
    if (!sdt.at(pm, c, pr, uc.factor)) {
      if (NEXT == 2) dt_inv = smax(untouched_cfl<D>(m, w, c), dt_inv);
      if (NEXT == 3) problem_cfl(pm, pr, untouched_cfl<D>(m, w, c));
      continue;
    }
    float shi[D + 2], slo[D + 2];
#pragma unroll
    for (int k = 0; k < D + 2; ++k) shi[k] = slo[k] = 0.f;
    const int q0 = m.cell_face_offsets[c], nq = m.cell_face_offsets[c + 1] - q0;
    for (int k = 0; k < nq; ++k) {
      const int sf = m.cell_faces[q0 + k];
      const int f = sf < 0 ? ~sf : sf;
      float F[4 * F4];
#pragma unroll
      for (int r = 0; r < F4; ++r) {
        const float4 t = w.fflux[(size_t)F4 * f + r];
        F[4 * r] = t.x;
        F[4 * r + 1] = t.y;
        F[4 * r + 2] = t.z;
        F[4 * r + 3] = t.w;
      }
#pragma unroll
      for (int k = 0; k < D + 2; ++k) two_sum_acc(shi[k], slo[k], sf >= 0 ? -F[k] : F[k]);
    }
    float vn[D], an;
    cell_update<D, STAGE>(s, w, pk_out, pm, c, pr, sdt.dts, shi, slo, uc, vn, &an,
                          STAGE == 1 && has_out ? &out : nullptr);
    if (NEXT == 2) dt_inv = smax(cell_cfl<D>(m, w, c, vn, an), dt_inv);
    if (NEXT == 3) problem_cfl(pm, pr, cell_cfl<D>(m, w, c, vn, an));
  }
  if (NEXT == 2) finish_cfl(w, nd, dt_inv);
}

// Colour schedule, part 1 (one launch per colour): one flux per face of the
// colour, subtracted from / added to its cells' compensated sums.  No two
// faces of a colour share a cell, so the read-modify-writes do not race; a
// cell receives its faces in colour order (deterministic, but not the cell's
// face order of the gather schedules, so the sums round differently).
template <int D, int KIND, bool SECOND, int BS>
__global__ void __launch_bounds__(BS, 1024 / BS)
face_colour_kernel(const fvh_mesh_view m, workspace w, const float4 *__restrict__ pk_in,
                   int swap, int outflow, int first, int count) {
  constexpr int NQ = D + 2;
  for (int i = blockIdx.x * BS + threadIdx.x; i < count; i += gridDim.x * BS) {
    const int f = w.colour_faces[first + i];
    float F[NQ];
    face_flux_area<D, KIND, SECOND>(m, w, pk_in, f, swap, outflow, F);
    const int2 cc = reinterpret_cast<const int2 *>(m.face_cells)[f];
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const int c = side == 0 ? cc.x : cc.y;
      if (c < 0) continue;
      float *a = w.acc + (size_t)2 * NQ * c;
#pragma unroll
      for (int k = 0; k < NQ; ++k) {
        float hi = a[k], lo = a[NQ + k];
        two_sum_acc(hi, lo, side == 0 ? -F[k] : F[k]);
        a[k] = hi;
        a[NQ + k] = lo;
      }
    }
  }
}

// Colour schedule, part 2: each cell takes its sums (and clears them for the
// next stage), then the update of the gather schedules.
template <int D, int BS, int STAGE, int NEXT = 0>
__global__ void __launch_bounds__(BS, 1024 / BS)
colour_update_kernel(const fvh_mesh_view m, const fvh_state_view s, workspace w,
                     float4 *__restrict__ pk_out, const problem_map pm,
                     const update_consts uc, int rev, const next_dt nd,
                     const fvh_state_view out, int has_out) {
  constexpr int NQ = D + 2;
  stage_dt sdt;
  float dt_inv = 0.f;
  for (int i = blockIdx.x * BS + threadIdx.x; i < m.num_cells; i += gridDim.x * BS) {
    const int c = rev ? m.num_cells - 1 - i : i;
    const int pr = pm.cell_problem ? pm.cell_problem[c] : 0;
    float *a = w.acc + (size_t)2 * NQ * c;
    float shi[NQ], slo[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      shi[k] = a[k];
      slo[k] = a[NQ + k];
      a[k] = a[NQ + k] = 0.f;
    }
    if (!sdt.at(pm, c, pr, uc.factor)) {
      if (NEXT == 2) dt_inv = smax(untouched_cfl<D>(m, w, c), dt_inv);
      continue;
    }
    float vn[D], an;
    cell_update<D, STAGE>(s, w, pk_out, pm, c, pr, sdt.dts, shi, slo, uc, vn, &an,
                          STAGE == 1 && has_out ? &out : nullptr);
    if (NEXT == 2) dt_inv = smax(cell_cfl<D>(m, w, c, vn, an), dt_inv);
  }
  if (NEXT == 2) finish_cfl(w, nd, dt_inv);
}

// Diagnostic: the integer-pipe conversions applied to an array, so they can be
// compared with exact host conversions.
__global__ void split_kernel(const double *x, int64_t n, float *hi, float *lo, float *h2,
                             double *back) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const df d = df_from(x[i]);
    hi[i] = d.hi;
    lo[i] = d.lo;
    h2[i] = d2f(x[i]);
    back[i] = f2d(d.hi);
  }
}

cudaError_t debug_split(const double *x, int64_t n, float *hi, float *lo, float *h2,
                        double *back, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int64_t nb = (n + 255) / 256;
  split_kernel<<<(int)(nb < 4096 ? nb : 4096), 256, 0, st>>>(x, n, hi, lo, h2, back);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <int D>
static size_t bytes_for(int nc, int nf, int nv) {
  using L = layout<D>;
  return sizeof(float4) * ((size_t)nc * (2 * L::PACK4 + L::GRAD4 + L::CEN4) + (size_t)nv * L::CEN4 +
                           (size_t)nf * (L::FGEO4 + L::FDX4 + L::FLUX4) + (size_t)nc * L::DEL4) +
         2 * sizeof(float) * (size_t)nc +
         256 * 18;  // alignment of each carved array + counters
}

template <int D>
static void carve(workspace *w) {
  using L = layout<D>;
  char *b = static_cast<char *>(w->base);
  auto take = [&](size_t bytes) {
    char *r = b;
    b += (bytes + 255) / 256 * 256;
    return r;
  };
  w->pack = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nc * L::PACK4));
  w->pack2 = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nc * L::PACK4));
  w->grads = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nc * L::GRAD4));
  w->ccen = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nc * L::CEN4));
  w->vcoord = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nv * L::CEN4));
  w->fgeo = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nf * L::FGEO4));
  w->fdx = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nf * L::FDX4));
  w->fflux = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nf * L::FLUX4));
  w->delta = reinterpret_cast<float4 *>(take(sizeof(float4) * (size_t)w->nc * L::DEL4));
  w->inv_vol32 = reinterpret_cast<float *>(take(sizeof(float) * (size_t)w->nc));
  w->inv_vol_lo = reinterpret_cast<float *>(take(sizeof(float) * (size_t)w->nc));
  w->ticket = reinterpret_cast<unsigned *>(take(256));
  w->dtinv_max = reinterpret_cast<unsigned *>(take(256));
}

template <int D>
static cudaError_t setup_d(const fvh_mesh_view &m, workspace *w, cudaStream_t st) {
  const int t = 256;
  setup_cells<D><<<(m.num_cells + t - 1) / t, t, 0, st>>>(m, *w);
  setup_vertices<D><<<(m.num_vertices + t - 1) / t, t, 0, st>>>(m, *w);
  setup_faces<D><<<(m.num_faces + t - 1) / t, t, 0, st>>>(m, *w);
  return cudaGetLastError();
}

cudaError_t setup_geometry(workspace *w, const fvh_mesh_view &m, cudaStream_t st) {
  if (m.num_cells > w->nc || m.num_faces > w->nf || m.num_vertices > w->nv)
    return cudaErrorInvalidValue;
  return m.dim == 2 ? setup_d<2>(m, w, st) : setup_d<3>(m, w, st);
}

fvh_status create_capacity(int dim, int64_t cells, int64_t faces, int64_t vertices,
                           workspace **out) {
  *out = nullptr;
  if ((dim != 2 && dim != 3) || cells <= 0 || faces <= 0 || vertices <= 0 ||
      cells > INT32_MAX || faces > INT32_MAX || vertices > INT32_MAX)
    return FVH_ERR_INVALID_ARGUMENT;
  workspace *w = new (std::nothrow) workspace();
  if (!w) return FVH_ERR_OUT_OF_MEMORY;
  w->dim = dim;
  w->nc = (int)cells;
  w->nf = (int)faces;
  w->nv = (int)vertices;
  const size_t bytes = dim == 2 ? bytes_for<2>(w->nc, w->nf, w->nv) : bytes_for<3>(w->nc, w->nf, w->nv);
  cudaError_t e = cudaMalloc(&w->base, bytes);
  if (e == cudaSuccess) e = cudaMemset(w->base, 0, bytes);
  if (e != cudaSuccess) {
    destroy(w);
    return e == cudaErrorMemoryAllocation ? FVH_ERR_OUT_OF_MEMORY : FVH_ERR_CUDA;
  }
  if (dim == 2)
    carve<2>(w);
  else
    carve<3>(w);
  *out = w;
  return FVH_OK;
}

// Greedy face colouring on the host (faces in id order, the smallest colour
// neither cell uses yet) for the colour schedule; deterministic.  A failed host
// allocation is reported as cudaErrorMemoryAllocation, not thrown.
static cudaError_t setup_colours_host(workspace *w, const fvh_mesh_view &m);
static cudaError_t setup_colours(workspace *w, const fvh_mesh_view &m) {
  try {
    return setup_colours_host(w, m);
  } catch (const std::bad_alloc &) {
    return cudaErrorMemoryAllocation;
  }
}
static cudaError_t setup_colours_host(workspace *w, const fvh_mesh_view &m) {
  std::vector<int32_t> fc(2 * (size_t)m.num_faces);
  cudaError_t e = cudaMemcpy(fc.data(), m.face_cells, sizeof(int32_t) * fc.size(),
                             cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  std::vector<uint32_t> used(m.num_cells, 0u);
  std::vector<int> colour(m.num_faces);
  int nc = 0;
  for (int f = 0; f < m.num_faces; ++f) {
    const int a = fc[2 * (size_t)f], b = fc[2 * (size_t)f + 1];
    const uint32_t taken = used[a] | (b >= 0 ? used[b] : 0u);
    int col = 0;
    while (col < kMaxColours && (taken >> col) & 1u) ++col;
    if (col == kMaxColours) return cudaErrorNotSupported;  // more than 32 colours
    colour[f] = col;
    used[a] |= 1u << col;
    if (b >= 0) used[b] |= 1u << col;
    nc = col + 1 > nc ? col + 1 : nc;
  }
  std::vector<int> off(nc + 1, 0), faces(m.num_faces);
  for (int f = 0; f < m.num_faces; ++f) off[colour[f] + 1]++;
  for (int k = 0; k < nc; ++k) off[k + 1] += off[k];
  std::vector<int> pos(off.begin(), off.end() - 1);
  for (int f = 0; f < m.num_faces; ++f) faces[pos[colour[f]]++] = f;
  w->ncolours = nc;
  for (int k = 0; k <= nc; ++k) w->colour_off[k] = off[k];
  const int NQ = w->dim + 2;
  e = cudaMalloc(&w->colour_faces, sizeof(int) * (size_t)m.num_faces);
  if (e == cudaSuccess) e = cudaMalloc(&w->acc, sizeof(float) * 2 * NQ * (size_t)m.num_cells);
  if (e == cudaSuccess)
    e = cudaMemcpy(w->colour_faces, faces.data(), sizeof(int) * faces.size(),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(w->acc, 0, sizeof(float) * 2 * NQ * (size_t)m.num_cells);
  return e;
}

bool staging(const workspace *w) { return w && w->stage.nchunks > 0; }

int colours(const workspace *w) { return w ? w->ncolours : 0; }

// Tables of the staged 2D gradients (see gradients_staged_kernel), built on
// the host from the mesh.  Chunks: kStageCells consecutive cells of the Morton
// order of the centroids (16-bit quantised coordinates, bits interleaved).
// Per chunk, a topology block of 32-bit words: 16-bit entry i of the first
// kStageCells / 2 words is the word offset of cell i's record (or 0xffff); a
// record is a word (own slot | nn << 8 | nr << 16), then the nn neighbour
// slots and the nr vertex slots, a byte each and four to a word -- a chunk
// stages at most 256 cell and 256 vertex records, so a slot fits in a byte.
// The stage buffers are sized for the mesh's largest chunk; a mesh with a
// chunk that does not fit keeps the global-memory kernel (nchunks stays 0).
static unsigned spread_bits16(unsigned x) {
  x &= 0xffffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

static cudaError_t setup_stage_host(workspace *w, const fvh_mesh_view &m) {
  const int nc = m.num_cells;
  std::vector<int> nb_off(nc + 1), cv_off(nc + 1);
  std::vector<double> cx(nc), cy(nc);
  cudaError_t e = cudaMemcpy(nb_off.data(), m.cell_nbr_offsets, sizeof(int) * (nc + 1),
                             cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(cv_off.data(), m.cell_vertex_offsets, sizeof(int) * (nc + 1),
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(cx.data(), m.cell_centroid[0], sizeof(double) * nc, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(cy.data(), m.cell_centroid[1], sizeof(double) * nc, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  std::vector<int> nb(nb_off[nc]), cv(cv_off[nc]);
  if (!nb.empty())
    e = cudaMemcpy(nb.data(), m.cell_nbrs, sizeof(int) * nb.size(), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && !cv.empty())
    e = cudaMemcpy(cv.data(), m.cell_vertices, sizeof(int) * cv.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  // Morton order of the centroids
  double x0 = cx[0], x1 = cx[0], y0 = cy[0], y1 = cy[0];
  for (int c = 0; c < nc; ++c) {
    x0 = std::min(x0, cx[c]); x1 = std::max(x1, cx[c]);
    y0 = std::min(y0, cy[c]); y1 = std::max(y1, cy[c]);
  }
  const double sx = x1 > x0 ? 65535.0 / (x1 - x0) : 0.0, sy = y1 > y0 ? 65535.0 / (y1 - y0) : 0.0;
  std::vector<std::pair<unsigned, int>> order(nc);
  for (int c = 0; c < nc; ++c) {
    const unsigned qx = (unsigned)((cx[c] - x0) * sx), qy = (unsigned)((cy[c] - y0) * sy);
    order[c] = {spread_bits16(qx) | (spread_bits16(qy) << 1), c};
  }
  std::sort(order.begin(), order.end());
  const int nchunks = (nc + kStageCells - 1) / kStageCells;
  std::vector<std::vector<stage_run>> runs(nchunks);
  std::vector<std::vector<unsigned>> topo(nchunks);
  int fits = 1, max_cells = 0, max_verts = 0, max_topo = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(& : fits) \
    reduction(max : max_cells, max_verts, max_topo)
  for (int k = 0; k < nchunks; ++k) {
    const int i0 = k * kStageCells, i1 = std::min(nc, i0 + kStageCells);
    std::vector<int> ids, vids;
    for (int i = i0; i < i1; ++i) {
      const int c = order[i].second;
      ids.push_back(c);
      for (int q = nb_off[c]; q < nb_off[c + 1]; ++q) ids.push_back(nb[q]);
      for (int r = cv_off[c]; r < cv_off[c + 1]; ++r) vids.push_back(cv[r]);
    }
    std::sort(ids.begin(), ids.end());
    ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
    std::sort(vids.begin(), vids.end());
    vids.erase(std::unique(vids.begin(), vids.end()), vids.end());
    if ((int)ids.size() > kStageMaxCells || (int)vids.size() > kStageMaxVerts) {
      fits = 0;
      continue;
    }
    auto add_runs = [&](const std::vector<int> &v, int kind) {
      for (size_t i = 0; i < v.size();) {
        size_t j = i + 1;
        while (j < v.size() && v[j] == v[j - 1] + 1) ++j;
        runs[k].push_back({v[i], (int)(j - i), (int)i, kind});
        i = j;
      }
    };
    add_runs(ids, 0);
    add_runs(vids, 1);
    auto pos = [](const std::vector<int> &v, int x) {
      return (unsigned)(std::lower_bound(v.begin(), v.end(), x) - v.begin());
    };
    constexpr int kIndexWords = kStageCells / 2;
    std::vector<unsigned> words(kIndexWords, 0xffffffffu);
    bool ok = true;
    for (int i = i0; i < i1 && ok; ++i) {
      const int c = order[i].second;
      const int nn = nb_off[c + 1] - nb_off[c], nr = cv_off[c + 1] - cv_off[c];
      ok = nn < 256 && nr < 256 && words.size() < 0xffffu;
      const unsigned at = (unsigned)words.size();
      unsigned &slot = words[(i - i0) / 2];
      slot = (i - i0) % 2 == 0 ? ((slot & 0xffff0000u) | at) : ((slot & 0xffffu) | (at << 16));
      words.push_back((unsigned)pos(ids, c) | ((unsigned)nn << 8) | ((unsigned)nr << 16));
      auto put_bytes = [&](const int *v, int n, const std::vector<int> &set) {
        for (int j = 0; j < n; j += 4) {
          unsigned wd = 0;
          for (int b = 0; b < 4 && j + b < n; ++b) wd |= (unsigned)pos(set, v[j + b]) << (8 * b);
          words.push_back(wd);
        }
      };
      put_bytes(nb.data() + nb_off[c], nn, ids);
      put_bytes(cv.data() + cv_off[c], nr, vids);
    }
    while (words.size() % 4) words.push_back(0);  // 16-byte multiple
    if (!ok) {
      fits = 0;
      continue;
    }
    max_cells = std::max(max_cells, (int)ids.size());
    max_verts = std::max(max_verts, (int)vids.size());
    max_topo = std::max(max_topo, (int)(4 * words.size()));
    topo[k] = std::move(words);
  }
  if (!fits) return cudaSuccess;  // the global-memory kernel serves this mesh
  auto up128 = [](int b) { return (b + 127) / 128 * 128; };
  stage_tables t;
  t.cen_at = up128(32 * max_cells);
  t.vtx_at = t.cen_at + up128(16 * max_cells);
  t.topo_at = t.vtx_at + up128(16 * max_verts);
  t.stage_bytes = t.topo_at + up128(max_topo);
  if (t.stage_bytes > kStageMaxBytes) return cudaSuccess;
  std::vector<int> cells((size_t)nchunks * kStageCells, -1);
  for (int i = 0; i < nc; ++i) cells[i] = order[i].second;
  std::vector<int> run_off(nchunks + 1, 0);
  std::vector<long long> topo_off(nchunks + 1, 0);
  std::vector<unsigned> chunk_bytes(nchunks, 0);
  for (int k = 0; k < nchunks; ++k) {
    run_off[k + 1] = run_off[k] + (int)runs[k].size();
    topo_off[k + 1] = topo_off[k] + 4 * (long long)topo[k].size();
    chunk_bytes[k] = 4 * (unsigned)topo[k].size();
    for (const stage_run &r : runs[k]) chunk_bytes[k] += (unsigned)r.count * (r.kind == 0 ? 48u : 16u);
  }
  std::vector<stage_run> all(run_off[nchunks]);
  std::vector<unsigned> blob(topo_off[nchunks] / 4);
  for (int k = 0; k < nchunks; ++k) {
    std::copy(runs[k].begin(), runs[k].end(), all.begin() + run_off[k]);
    std::copy(topo[k].begin(), topo[k].end(), blob.begin() + topo_off[k] / 4);
  }
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t b_cells = up(sizeof(int) * cells.size()), b_off = up(sizeof(int) * run_off.size()),
               b_runs = up(sizeof(stage_run) * all.size()),
               b_toff = up(sizeof(long long) * topo_off.size()),
               b_topo = up(sizeof(unsigned) * blob.size()),
               b_bytes = up(sizeof(unsigned) * chunk_bytes.size());
  char *base = nullptr;
  e = cudaMalloc(&base, b_cells + b_off + b_runs + b_toff + b_topo + b_bytes);
  if (e != cudaSuccess) return e;
  w->stage_base = base;
  char *p = base;
  auto put = [&](const void *src, size_t bytes, size_t span) {
    char *d = p;
    if (e == cudaSuccess && bytes) e = cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice);
    p += span;
    return d;
  };
  t.nchunks = nchunks;
  t.cells = reinterpret_cast<const int *>(put(cells.data(), sizeof(int) * cells.size(), b_cells));
  t.run_off = reinterpret_cast<const int *>(put(run_off.data(), sizeof(int) * run_off.size(), b_off));
  t.runs = reinterpret_cast<const stage_run *>(put(all.data(), sizeof(stage_run) * all.size(), b_runs));
  t.topo_off = reinterpret_cast<const long long *>(
      put(topo_off.data(), sizeof(long long) * topo_off.size(), b_toff));
  t.topo = reinterpret_cast<const unsigned *>(put(blob.data(), sizeof(unsigned) * blob.size(), b_topo));
  t.bytes = reinterpret_cast<const unsigned *>(
      put(chunk_bytes.data(), sizeof(unsigned) * chunk_bytes.size(), b_bytes));
  if (e != cudaSuccess) return e;
  // persistent grid: the blocks that fit on the device at once
  const int smem = 2 * t.stage_bytes;
  e = cudaFuncSetAttribute(gradients_staged_kernel<true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(gradients_staged_kernel<false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int per_sm = 0, dev = 0, sms = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gradients_staged_kernel<true>,
                                                      kStageCells, smem);
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess || per_sm < 1) return e;
  w->stage = t;
  w->stage_blocks = std::min(nchunks, per_sm * sms);
  return cudaSuccess;
}

static cudaError_t setup_stage(workspace *w, const fvh_mesh_view &m) {
  if (m.dim != 2) return cudaSuccess;
  try {
    return setup_stage_host(w, m);
  } catch (const std::bad_alloc &) {
    return cudaErrorMemoryAllocation;
  }
}

fvh_status create(const fvh_mesh_view &m, const fvh_params &p, workspace **out) {
  (void)p;
  const fvh_status r = create_capacity(m.dim, m.num_cells, m.num_faces, m.num_vertices, out);
  if (r != FVH_OK) return r;
  cudaError_t e = setup_geometry(*out, m, nullptr);
  if (e == cudaSuccess) e = setup_colours(*out, m);
  if (e == cudaSuccess) e = setup_stage(*out, m);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    destroy(*out);
    *out = nullptr;
    return e == cudaErrorMemoryAllocation ? FVH_ERR_OUT_OF_MEMORY : FVH_ERR_CUDA;
  }
  return FVH_OK;
}

void destroy(workspace *w) {
  if (!w) return;
  cudaFree(w->stage_base);
  cudaFree(w->colour_faces);
  cudaFree(w->acc);
  cudaFree(w->base);
  delete w;
}

template <int D, int KIND, bool SECOND, int BS>
// dir: traversal direction of the previous launch; each launch runs the other
// way, so it starts on the cells/faces its predecessor touched last (still in
// L2).  Results do not depend on the order.
static void launch_stage_bs(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                            const fvh_state_view &s, const problem_map &pm, int stage,
                            int cpt, int schedule, bool staged, cudaStream_t st,
                            const launch_mark &mark,
                            int &dir, const next_dt *nd) {
  const long long per = (long long)BS * cpt;
  const int nb = (int)((m.num_cells + per - 1) / per);
  const float4 *pk_in = stage == 0 ? w->pack : w->pack2;
  // nd is given for a single mesh (the batch has per-problem dt kernels)
  const bool next = stage == 1 && nd != nullptr && nd->write_next;
  float4 *pk_out = stage == 0 ? w->pack2 : next ? w->pack : nullptr;
  const next_dt ndv = nd ? *nd : next_dt();
  // a corrector that finishes dt ends with one same-address atomic pair per
  // block: at most kCflMaxBlocks blocks (grid-stride)
  const int nb_next = nb < kCflMaxBlocks ? nb : kCflMaxBlocks;
  if (SECOND) {
    dir ^= 1;
    if (D == 2 && staged && w->stage.nchunks > 0 && !pm.cell_problem) {
      const int smem = 2 * w->stage.stage_bytes;
      if (p.limiter == FVH_LIMITER_NONE)
        gradients_staged_kernel<false><<<w->stage_blocks, kStageCells, smem, st>>>(
            m, *w, pk_in, w->stage, dir, pm.status);
      else
        gradients_staged_kernel<true><<<w->stage_blocks, kStageCells, smem, st>>>(
            m, *w, pk_in, w->stage, dir, pm.status);
    } else if (p.limiter == FVH_LIMITER_NONE) {
      gradients_kernel<D, false, BS><<<nb, BS, 0, st>>>(m, *w, pk_in, dir);
    } else {
      gradients_kernel<D, true, BS><<<nb, BS, 0, st>>>(m, *w, pk_in, dir);
    }
    mark("gradients");
  }
  update_consts k;
  const double gm1 = p.gamma - 1.0;
  k.gm1.hi = (float)gm1;
  k.gm1.lo = (float)(gm1 - (double)k.gm1.hi);
  k.ggm1 = (float)(p.gamma * (p.gamma - 1.0));
  k.factor = 0.5f;
  k.inv_cv = 1.0 / p.cv;
  k.unit_cv = p.cv == 1.0;
  if (schedule == 2) {
    for (int col = 0; col < w->ncolours; ++col) {
      const int first = w->colour_off[col], count = w->colour_off[col + 1] - first;
      const int nbc = (int)((count + per - 1) / per);
      face_colour_kernel<D, KIND, SECOND, BS><<<nbc > 0 ? nbc : 1, BS, 0, st>>>(
          m, *w, pk_in, p.recon_swap_ep, p.boundary, first, count);
      mark("face_colour");
    }
    dir ^= 1;
    if (stage == 0)
      colour_update_kernel<D, BS, 0><<<nb, BS, 0, st>>>(m, s, *w, pk_out, pm, k, dir, ndv,
                                                        ndv.out, 0);
    else if (next)
      colour_update_kernel<D, BS, 1, 2><<<nb_next, BS, 0, st>>>(m, s, *w, pk_out, pm, k, dir,
                                                                 ndv, ndv.out, ndv.has_out);
    else
      colour_update_kernel<D, BS, 1><<<nb, BS, 0, st>>>(m, s, *w, pk_out, pm, k, dir, ndv,
                                                        ndv.out, ndv.has_out);
    mark("colour_update");
  } else if (schedule == 1) {
    const int nbf = (int)((m.num_faces + per - 1) / per);
    dir ^= 1;
    face_flux_kernel<D, KIND, SECOND, BS><<<nbf, BS, 0, st>>>(m, *w, pk_in, p.recon_swap_ep,
                                                               p.boundary, dir);
    mark("face_flux");
    dir ^= 1;
    if (stage == 0)
      gather_update_kernel<D, BS, 0><<<nb, BS, 0, st>>>(m, s, *w, pk_out, pm, k, dir, ndv,
                                                        ndv.out, 0);
    else if (next && ndv.batch)
      gather_update_kernel<D, BS, 1, 3><<<nb, BS, 0, st>>>(m, s, *w, pk_out, pm, k, dir, ndv,
                                                           ndv.out, ndv.has_out);
    else if (next)
      gather_update_kernel<D, BS, 1, 2><<<nb_next, BS, 0, st>>>(m, s, *w, pk_out, pm, k, dir,
                                                                 ndv, ndv.out, ndv.has_out);
    else
      gather_update_kernel<D, BS, 1><<<nb, BS, 0, st>>>(m, s, *w, pk_out, pm, k, dir, ndv,
                                                        ndv.out, ndv.has_out);
    mark("gather_update");
  } else {
    dir ^= 1;
    if (stage == 0)
      flux_update_kernel<D, KIND, SECOND, BS, 0><<<nb, BS, 0, st>>>(
          m, s, *w, pk_in, pk_out, pm, k, p.recon_swap_ep, p.boundary, dir, ndv, ndv.out, 0);
    else if (next && ndv.batch)
      flux_update_kernel<D, KIND, SECOND, BS, 1, 3><<<nb, BS, 0, st>>>(
          m, s, *w, pk_in, pk_out, pm, k, p.recon_swap_ep, p.boundary, dir, ndv, ndv.out,
          ndv.has_out);
    else if (next)
      flux_update_kernel<D, KIND, SECOND, BS, 1, 2><<<nb_next, BS, 0, st>>>(
          m, s, *w, pk_in, pk_out, pm, k, p.recon_swap_ep, p.boundary, dir, ndv, ndv.out,
          ndv.has_out);
    else
      flux_update_kernel<D, KIND, SECOND, BS, 1><<<nb, BS, 0, st>>>(
          m, s, *w, pk_in, pk_out, pm, k, p.recon_swap_ep, p.boundary, dir, ndv, ndv.out,
          ndv.has_out);
    mark("flux_update");
  }
}

template <int D, int KIND, bool SECOND>
static void launch_stage(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                         const fvh_state_view &s, const problem_map &pm, int stage,
                         const launch_shape &sh, cudaStream_t st, const launch_mark &mark,
                         int &dir, const next_dt *nd) {
  if (sh.block == 256)
    launch_stage_bs<D, KIND, SECOND, 256>(w, m, p, s, pm, stage, sh.cells_per_thread,
                                          sh.schedule, sh.staged, st, mark, dir, nd);
  else
    launch_stage_bs<D, KIND, SECOND, 128>(w, m, p, s, pm, stage, sh.cells_per_thread,
                                          sh.schedule, sh.staged, st, mark, dir, nd);
}

template <int D, int KIND>
static void launch_stage_k(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                           const fvh_state_view &s, const problem_map &pm, int stage,
                           const launch_shape &sh, cudaStream_t st, const launch_mark &mark,
                           int &dir, const next_dt *nd) {
  if (p.order == 1)
    launch_stage<D, KIND, false>(w, m, p, s, pm, stage, sh, st, mark, dir, nd);
  else
    launch_stage<D, KIND, true>(w, m, p, s, pm, stage, sh, st, mark, dir, nd);
}

template <int D>
static void launch_stages(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                          const fvh_state_view &s, const problem_map &pm,
                          const launch_shape &sh, cudaStream_t st, const launch_mark &mark,
                          int dir, const next_dt *nd = nullptr) {
  for (int stage = 0; stage < 2; ++stage) {
    if (p.flux_kind == FVH_FLUX_RUSANOV)
      launch_stage_k<D, FVH_FLUX_RUSANOV>(w, m, p, s, pm, stage, sh, st, mark, dir, nd);
    else if (p.flux_kind == FVH_FLUX_HLLC)
      launch_stage_k<D, FVH_FLUX_HLLC>(w, m, p, s, pm, stage, sh, st, mark, dir, nd);
    else
      launch_stage_k<D, FVH_FLUX_HLLE>(w, m, p, s, pm, stage, sh, st, mark, dir, nd);
  }
}

template <int D>
static cudaError_t step_d(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                          const fvh_state_view &s, double *t, double *dt, double *partial,
                          int dt_blocks, fvh_device_status *status, cudaStream_t st,
                          const launch_mark &mark, const launch_shape &shape,
                          const step_flags &f) {
  if (f.pack_first) {
    pack_dt_kernel<D><<<dt_blocks, kDtThreads, 0, st>>>(m, s, *w, partial, p, t, dt, status, 0,
                                                         f.src ? *f.src : s, f.src ? 1 : 0);
    mark("pack_dt");
  }
  problem_map pm;
  pm.dt = dt;
  pm.t = t;
  pm.status = status;
  next_dt nd;
  nd.cfl = p.cfl;
  nd.final_time = p.final_time;
  nd.soln_time = t;
  nd.dt = dt;
  nd.status = status;
  nd.write_next = f.write_next;
  if (f.out) {
    nd.out = *f.out;
    nd.has_out = 1;
  }
  // pack_dt and every corrector run upwards, so the gradients start downwards
  launch_stages<D>(w, m, p, s, pm, shape, st, mark, 0, &nd);
  return cudaGetLastError();
}

cudaError_t step(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                 const fvh_state_view &s, double *soln_time, double *dt, double *partial,
                 int dt_blocks, fvh_device_status *status, cudaStream_t st,
                 const launch_mark &mark, const launch_shape &shape, step_flags f) {
  return m.dim == 2
             ? step_d<2>(w, m, p, s, soln_time, dt, partial, dt_blocks, status, st, mark, shape, f)
             : step_d<3>(w, m, p, s, soln_time, dt, partial, dt_blocks, status, st, mark, shape, f);
}

template <int D>
static cudaError_t step_batch_d(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                                const fvh_state_view &s, const problem_map &pm,
                                const launch_shape &sh, cudaStream_t st,
                                const launch_mark &mark, const step_flags &f) {
  if (f.pack_first) {
    const int nb = (m.num_cells + kDtThreads - 1) / kDtThreads;
    pack_dt_batch_kernel<D><<<nb, kDtThreads, 0, st>>>(m, s, *w, pm, 0);
    mark("pack_dt");
  }
  dt_final_batch_kernel<<<(pm.nproblems + 127) / 128, 128, 0, st>>>(pm, 0);
  mark("dt_final");
  next_dt nd;
  nd.write_next = f.write_next;
  nd.batch = 1;
  launch_stages<D>(w, m, p, s, pm, sh, st, mark, 0, &nd);
  return cudaGetLastError();
}

cudaError_t step_batch(workspace *w, const fvh_mesh_view &m, const fvh_params &p,
                       const fvh_state_view &s, const problem_map &pm,
                       const launch_shape &shape, cudaStream_t st, const launch_mark &mark,
                       step_flags f) {
  return m.dim == 2 ? step_batch_d<2>(w, m, p, s, pm, shape, st, mark, f)
                    : step_batch_d<3>(w, m, p, s, pm, shape, st, mark, f);
}

int launches_per_step(const fvh_params &p, const launch_shape &sh, step_flags f,
                      int ncolours) {
  const int fluxes = sh.schedule == 2 ? ncolours + 1 : sh.schedule == 1 ? 2 : 1;
  const int per_stage = (p.order == 1 ? 0 : 1) + fluxes;
  return (f.pack_first ? 1 : 0) + 2 * per_stage;
}

int launches_per_step_batch(const fvh_params &p, const launch_shape &sh, step_flags f) {
  return launches_per_step(p, sh, f) + 1;  // per-problem dt is a separate kernel
}

int launches_per_step(const fvh_params &p) { return launches_per_step(p, launch_shape()); }

}  // namespace mixed
}  // namespace fvh
