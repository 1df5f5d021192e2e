"""ORACLE — test infrastructure only (see hydro_oracle.cpp).

Loads liboracle_hydro.so, the CPU restatement of the reference hydro tasks,
plus an independent builder of the benchmark's structured box mesh
(box_mesh.cpp).  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs
use it, always as the checker or the timed CPU baseline, never as the product
path.  It never imports or loads the product library: its ctypes structures
are declared here from the C header's layout (include/flecsale_gb300.h), and
its entry points take the structures as untyped pointers, so views built by
the product's binding can be passed too.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "liboracle_hydro.so")
SOURCES = [os.path.join(HERE, "hydro_oracle.cpp"), os.path.join(HERE, "box_mesh.cpp")]
_L = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)

# fvh_flux_kind / fvh_limiter_kind / fvh_boundary_kind values of the C header
FLUX = {"hlle": 0, "rusanov": 1, "hllc": 2}
LIMITER = {"barth_jespersen": 0, "none": 1}
BOUNDARY = {"wall": 0, "outflow": 1}


class Params(C.Structure):
    """fvh_params (include/flecsale_gb300.h)."""
    _fields_ = [("dim", C.c_int32), ("flux_kind", C.c_int32), ("limiter", C.c_int32),
                ("order", C.c_int32), ("recon_swap_ep", C.c_int32), ("precision", C.c_int32),
                ("boundary", C.c_int32), ("reserved", C.c_int32), ("gamma", C.c_double),
                ("cv", C.c_double), ("cfl", C.c_double), ("final_time", C.c_double)]


class MeshView(C.Structure):
    """fvh_mesh_view (include/flecsale_gb300.h)."""
    _fields_ = [("dim", C.c_int32), ("num_cells", C.c_int32), ("num_faces", C.c_int32),
                ("num_vertices", C.c_int32),
                ("face_cells", _ip), ("cell_face_offsets", _ip), ("cell_faces", _ip),
                ("cell_nbr_offsets", _ip), ("cell_nbrs", _ip),
                ("cell_vertex_offsets", _ip), ("cell_vertices", _ip),
                ("cell_centroid", _dp * 3), ("cell_volume", _dp),
                ("face_centroid", _dp * 3), ("face_normal", _dp * 3), ("face_area", _dp),
                ("vertex_coord", _dp * 3)]


class StateView(C.Structure):
    """fvh_state_view (include/flecsale_gb300.h)."""
    _fields_ = [("density", _dp), ("velocity", _dp * 3), ("internal_energy", _dp),
                ("pressure", _dp), ("temperature", _dp), ("sound_speed", _dp)]


def params(dim: int, flux: str = "hlle", limiter: str = "barth_jespersen", order: int = 2,
           swap: bool = True, gamma: float = 1.4, cv: float = 1.0, cfl: float | None = None,
           final_time: float = 0.2, boundary: str = "wall") -> Params:
    """The reference's defaults (apps/hydro/2d/inputs.cc:27-42; CFL 1/3 in 3D,
    3d/inputs.cc:108), FP64."""
    p = Params()
    p.dim, p.flux_kind, p.limiter, p.order = dim, FLUX[flux], LIMITER[limiter], order
    p.recon_swap_ep, p.precision, p.boundary = 1 if swap else 0, 0, BOUNDARY[boundary]
    p.gamma, p.cv = gamma, cv
    p.cfl = (1.0 / 3.0 if dim == 3 else 0.5) if cfl is None else cfl
    p.final_time = final_time
    return p


def state_view(planes: np.ndarray, dim: int) -> StateView:
    """View over host planes (d, v[dim], e, p, T, a) of shape (5 + dim, n)."""
    assert planes.dtype == np.float64 and planes.flags.c_contiguous and planes.shape[0] >= 5 + dim
    ptr = lambda r: planes[r].ctypes.data_as(_dp)
    s = StateView()
    s.density = ptr(0)
    for d in range(dim):
        s.velocity[d] = ptr(1 + d)
    s.internal_energy, s.pressure = ptr(1 + dim), ptr(2 + dim)
    s.temperature, s.sound_speed = ptr(3 + dim), ptr(4 + dim)
    return s


def build(force: bool = False) -> str:
    """g++ -O2 without floating-point contraction, OpenMP over cells/faces."""
    hdr = os.path.join(ROOT, "include", "flecsale_gb300.h")
    stale = (not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
        max(os.path.getmtime(s) for s in SOURCES), os.path.getmtime(hdr),
        os.path.getmtime(__file__)))
    if force or stale:
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared",
               "-fopenmp", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
               *SOURCES, "-o", LIB + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def load() -> C.CDLL:
    global _L
    if _L is None:
        L = C.CDLL(build())
        vp, dp, i64p = C.c_void_p, _dp, C.POINTER(C.c_int64)
        # mesh, state, gradient, flux and params arguments are pointers to the
        # C header's structures (this module's or the product binding's)
        L.oracle_evaluate_time_step.argtypes = [vp, vp, vp, C.c_double, dp]
        L.oracle_evaluate_time_step.restype = C.c_int
        L.oracle_evaluate_gradients.argtypes = [vp, vp, vp, vp]
        L.oracle_evaluate_gradients.restype = None
        L.oracle_evaluate_fluxes.argtypes = [vp, vp, vp, vp, vp]
        L.oracle_evaluate_fluxes.restype = None
        L.oracle_apply_update.argtypes = [vp, vp, C.c_double, C.c_double, vp, vp, dp, i64p]
        L.oracle_apply_update.restype = C.c_int
        L.oracle_set_threads.argtypes = [C.c_int32]
        L.oracle_set_threads.restype = None
        L.oracle_max_threads.argtypes = []
        L.oracle_max_threads.restype = C.c_int32
        L.oracle_run.argtypes = [vp, vp, vp, C.c_int64, C.c_int, dp, i64p, i64p]
        L.oracle_run.restype = C.c_int
        L.oracle_state_from_pressure.argtypes = [C.c_int32, C.c_double, C.c_double, dp, dp,
                                                 dp, dp, dp]
        L.oracle_state_from_pressure.restype = None
        L.oracle_face_flux.argtypes = [C.c_int32, C.c_int32, dp, dp, dp, dp]
        L.oracle_face_flux.restype = None
        L.oracle_update_cell.argtypes = [C.c_int32, C.c_double, C.c_double, dp, dp]
        L.oracle_update_cell.restype = None
        L.oracle_box2d_sizes.argtypes = [C.c_int32, C.c_int32, i64p, i64p, i64p, i64p]
        L.oracle_box2d_sizes.restype = None
        L.oracle_box2d_build.argtypes = ([C.c_int32, C.c_int32] + [C.c_double] * 5
                                         + [C.c_uint64] + [vp] * 13)
        L.oracle_box2d_build.restype = None
        _L = L
    return _L


class BoxMesh2D:
    """The nx x ny quad box on [lo, hi], interior vertices jittered (seeded),
    built by box_mesh.cpp; `view` is an fvh_mesh_view over its arrays."""

    def __init__(self, nx: int, ny: int, lo=(0.0, 0.0), hi=(1.0, 1.0), jitter: float = 0.0,
                 seed: int = 0):
        L = load()
        nv, nf, ncf, nnb = (C.c_int64() for _ in range(4))
        L.oracle_box2d_sizes(nx, ny, C.byref(nv), C.byref(nf), C.byref(ncf), C.byref(nnb))
        nc = nx * ny
        self.dim, self.num_cells, self.num_faces, self.num_vertices = 2, nc, nf.value, nv.value
        i32 = lambda n: np.zeros(n, np.int32)
        f64 = lambda *s: np.zeros(s, np.float64)
        a = {"face_cells": i32(2 * nf.value), "cell_face_offsets": i32(nc + 1),
             "cell_faces": i32(ncf.value), "cell_nbr_offsets": i32(nc + 1),
             "cell_nbrs": i32(nnb.value), "cell_vertex_offsets": i32(nc + 1),
             "cell_vertices": i32(4 * nc), "cell_centroid": f64(2, nc), "cell_volume": f64(nc),
             "face_centroid": f64(2, nf.value), "face_normal": f64(2, nf.value),
             "face_area": f64(nf.value), "vertex_coord": f64(2, nv.value)}
        order = ["face_cells", "cell_face_offsets", "cell_faces", "cell_nbr_offsets", "cell_nbrs",
                 "cell_vertex_offsets", "cell_vertices", "cell_centroid", "cell_volume",
                 "face_centroid", "face_normal", "face_area", "vertex_coord"]
        L.oracle_box2d_build(nx, ny, lo[0], lo[1], hi[0], hi[1], jitter, seed,
                             *[a[k].ctypes.data for k in order])
        self._a = a
        v = MeshView()
        v.dim, v.num_cells, v.num_faces, v.num_vertices = 2, nc, nf.value, nv.value
        for k in order[:7]:
            setattr(v, k, a[k].ctypes.data_as(_ip))
        v.cell_volume = a["cell_volume"].ctypes.data_as(_dp)
        v.face_area = a["face_area"].ctypes.data_as(_dp)
        for d in range(2):
            v.cell_centroid[d] = a["cell_centroid"][d].ctypes.data_as(_dp)
            v.face_centroid[d] = a["face_centroid"][d].ctypes.data_as(_dp)
            v.face_normal[d] = a["face_normal"][d].ctypes.data_as(_dp)
            v.vertex_coord[d] = a["vertex_coord"][d].ctypes.data_as(_dp)
        self.view = v

    def arrays(self) -> dict:
        return self._a


def four_quadrant_state(mesh: BoxMesh2D, gamma: float = 1.4, cv: float = 1.0) -> np.ndarray:
    """Four-quadrant Riemann problem (rho, u, v, p) by cell centroid: NE
    (1.5, 0, 0, 1.5), NW (0.5323, 1.206, 0, 0.3), SW (0.138, 1.206, 1.206,
    0.029), SE (0.5323, 0, 1.206, 0.3), split at x = 0.5 and y = 0.5; then the
    ideal-gas closure (flecsale/eos/ideal_gas.h:178-226).  Planes (d, u, v, e,
    p, T, a)."""
    x, y = mesh.arrays()["cell_centroid"]
    east, north = x >= 0.5, y >= 0.5
    nc = mesh.num_cells
    d, u, v, p = (np.empty(nc) for _ in range(4))
    for sel, st in (((east & north), (1.5, 0.0, 0.0, 1.5)), ((~east & north), (0.5323, 1.206, 0.0, 0.3)),
                    ((~east & ~north), (0.138, 1.206, 1.206, 0.029)),
                    ((east & ~north), (0.5323, 0.0, 1.206, 0.3))):
        d[sel], u[sel], v[sel], p[sel] = st
    out = np.zeros((7, nc))
    out[0], out[1], out[2], out[4] = d, u, v, p
    load().oracle_state_from_pressure(nc, gamma, cv, d.ctypes.data_as(_dp), p.ctypes.data_as(_dp),
                                      out[3].ctypes.data_as(_dp), out[5].ctypes.data_as(_dp),
                                      out[6].ctypes.data_as(_dp))
    return out


def run(mesh, state: np.ndarray, p: Params, nsteps: int, stop_at_final: bool = False,
        t: float = 0.0):
    """oracle_run on host planes; returns (status, time, steps)."""
    tt, n, bad = C.c_double(t), C.c_int64(), C.c_int64(-1)
    st = load().oracle_run(C.byref(mesh.view), C.byref(p), C.byref(state_view(state, mesh.dim)),
                           nsteps, 1 if stop_at_final else 0, C.byref(tt), C.byref(n), C.byref(bad))
    return st, tt.value, n.value
