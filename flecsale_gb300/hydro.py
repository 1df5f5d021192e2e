"""ctypes binding of libflecsale_gb300.so (include/flecsale_gb300.h).

The C++/CUDA library is the product; this module only marshals arguments for
Python callers (tests, benchmark, examples).  Importing it never falls back to
another implementation: if the shared library is missing it is built, and if it
cannot be built or loaded an error is raised.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

_LIB: Optional[C.CDLL] = None

# fvh_status
OK, ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_INFINITE_DT, ERR_NEGATIVE_STATE = 0, 1, 2, 3, 4
ERR_UNSUPPORTED, ERR_NO_DEVICE, ERR_OUT_OF_MEMORY, ERR_CAPACITY, ERR_TIMEOUT = 5, 6, 7, 8, 9
# fvh_flux_kind / fvh_limiter_kind / fvh_precision
FLUX = {"hlle": 0, "rusanov": 1, "hllc": 2}
LIMITER = {"barth_jespersen": 0, "none": 1}
PRECISION = {"fp64": 0, "mixed": 1}
BOUNDARY = {"wall": 0, "outflow": 1}
# fvh_problem_kind
PROBLEM = {"shock_box": 0, "sod": 1, "four_quadrant": 2, "inner_cube": 3,
           "kelvin_helmholtz": 4, "uniform": 5}
STATUS_CLEAR = (1 << 64) - 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class Params(C.Structure):
    _fields_ = [("dim", C.c_int32), ("flux_kind", C.c_int32), ("limiter", C.c_int32),
                ("order", C.c_int32), ("recon_swap_ep", C.c_int32), ("precision", C.c_int32),
                ("boundary", C.c_int32), ("reserved", C.c_int32), ("gamma", C.c_double), ("cv", C.c_double), ("cfl", C.c_double),
                ("final_time", C.c_double)]


class MeshView(C.Structure):
    _fields_ = [("dim", C.c_int32), ("num_cells", C.c_int32), ("num_faces", C.c_int32),
                ("num_vertices", C.c_int32),
                ("face_cells", _ip), ("cell_face_offsets", _ip), ("cell_faces", _ip),
                ("cell_nbr_offsets", _ip), ("cell_nbrs", _ip),
                ("cell_vertex_offsets", _ip), ("cell_vertices", _ip),
                ("cell_centroid", _dp * 3), ("cell_volume", _dp),
                ("face_centroid", _dp * 3), ("face_normal", _dp * 3), ("face_area", _dp),
                ("vertex_coord", _dp * 3)]


class StateView(C.Structure):
    _fields_ = [("density", _dp), ("velocity", _dp * 3), ("internal_energy", _dp),
                ("pressure", _dp), ("temperature", _dp), ("sound_speed", _dp)]


class GradientView(C.Structure):
    _fields_ = [("density", _dp * 3), ("velocity", (_dp * 3) * 3),
                ("internal_energy", _dp * 3), ("pressure", _dp * 3),
                ("sound_speed", _dp * 3)]


class FluxView(C.Structure):
    _fields_ = [("mass", _dp), ("momentum", _dp * 3), ("energy", _dp)]


def make_params(dim: int, flux: str = "hlle", limiter: str = "barth_jespersen",
                order: int = 2, swap: bool = True, precision: str = "fp64",
                gamma: float = 1.4, cv: float = 1.0, cfl: Optional[float] = None,
                final_time: float = 0.2, boundary: str = "wall") -> Params:
    """fvh_params; defaults are the reference's (apps/hydro/2d/inputs.cc:27-42)."""
    p = Params()
    lib().fvh_params_default(C.byref(p), dim)
    p.flux_kind = FLUX[flux]
    p.limiter = LIMITER[limiter]
    p.order = order
    p.recon_swap_ep = 1 if swap else 0
    p.precision = PRECISION[precision]
    p.boundary = BOUNDARY[boundary]
    p.gamma, p.cv = gamma, cv
    if cfl is not None:
        p.cfl = cfl
    p.final_time = final_time
    return p


def _declare(L: C.CDLL) -> None:
    vp, sz = C.c_void_p, C.c_size_t
    sig = {
        "fvh_status_string": (C.c_char_p, [C.c_int32]),
        "fvh_abi_version": (C.c_int32, []),
        "fvh_params_default": (None, [C.POINTER(Params), C.c_int32]),
        "fvh_status_decode": (None, [C.c_uint64, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
        "fvh_time_step_workspace_bytes": (sz, [C.c_int32]),
        "fvh_evaluate_time_step": (C.c_int, [C.POINTER(MeshView), C.POINTER(StateView),
                                             C.POINTER(Params), vp, vp, vp, sz, vp, vp]),
        "fvh_evaluate_gradients": (C.c_int, [C.POINTER(MeshView), C.POINTER(StateView),
                                             C.POINTER(GradientView), C.POINTER(Params), vp]),
        "fvh_evaluate_fluxes": (C.c_int, [C.POINTER(MeshView), C.POINTER(StateView),
                                          C.POINTER(GradientView), C.POINTER(FluxView),
                                          C.POINTER(Params), vp]),
        "fvh_apply_update": (C.c_int, [C.POINTER(MeshView), C.POINTER(Params), vp, C.c_double,
                                       C.POINTER(FluxView), C.POINTER(StateView), vp, vp, vp]),
        "fvh_solver_create": (C.c_int, [C.POINTER(MeshView), C.POINTER(Params),
                                        C.POINTER(vp)]),
        "fvh_solver_destroy": (None, [vp]),
        "fvh_solver_step": (C.c_int, [vp, C.POINTER(StateView), vp]),
        "fvh_solver_run": (C.c_int, [vp, C.POINTER(StateView), C.c_int64, C.c_int32, C.c_int32,
                                     C.POINTER(C.c_int64), vp]),
        "fvh_solver_soln_time": (vp, [vp]),
        "fvh_solver_dt": (vp, [vp]),
        "fvh_solver_status": (vp, [vp]),
        "fvh_solver_gradients": (C.POINTER(GradientView), [vp]),
        "fvh_solver_fluxes": (C.POINTER(FluxView), [vp]),
        "fvh_solver_check": (C.c_int, [vp, vp, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
        "fvh_solver_reset": (C.c_int, [vp, C.c_double, vp]),
        "fvh_host_mesh_create": (C.c_int, [C.c_int32, C.c_int32, _dp, C.c_int32, _ip, _ip,
                                           C.POINTER(vp)]),
        "fvh_host_mesh_box": (C.c_int, [C.c_int32, _ip, _dp, _dp, C.c_double, C.c_uint64,
                                        C.POINTER(vp)]),
        "fvh_host_mesh_destroy": (None, [vp]),
        "fvh_host_mesh_view": (C.c_int, [vp, C.POINTER(MeshView)]),
        "fvh_host_mesh_nnz": (C.c_int, [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                        C.POINTER(C.c_int64)]),
        "fvh_host_initial_state": (C.c_int, [C.c_int32, vp, C.POINTER(Params), C.c_uint64, _dp]),
        "fvh_device_mesh_create": (C.c_int, [vp, C.POINTER(vp)]),
        "fvh_device_mesh_destroy": (None, [vp]),
        "fvh_device_mesh_view": (C.POINTER(MeshView), [vp]),
        "fvh_device_state_create": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(vp)]),
        "fvh_device_state_destroy": (None, [vp]),
        "fvh_device_state_view": (C.POINTER(StateView), [vp]),
        "fvh_state_upload": (C.c_int, [C.POINTER(StateView), C.c_int32, C.c_int32, _dp, vp]),
        "fvh_state_download": (C.c_int, [C.POINTER(StateView), C.c_int32, C.c_int32, _dp, vp]),
        "fvh_solver_advance_host": (C.c_int, [vp, C.POINTER(StateView), _dp, C.c_int64,
                                              C.POINTER(C.c_double), vp]),
        "fvh_solver_launches_per_step": (C.c_int32, [vp]),
        "fvh_solver_set_shape": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int32]),
        "fvh_solver_launches_per_run": (C.c_int64, [vp, C.c_int64]),
        "fvh_debug_split": (C.c_int, [vp, C.c_int64, vp, vp, vp, vp, vp]),
        "fvh_debug_sf64": (C.c_int, [C.c_int32, vp, vp, C.c_int64, vp, vp]),
        "fvh_input_load": (C.c_int, [C.c_char_p, C.c_char_p, C.c_size_t, C.POINTER(vp)]),
        "fvh_input_load_string": (C.c_int, [C.c_char_p, C.c_char_p, C.c_size_t, C.POINTER(vp)]),
        "fvh_input_destroy": (None, [vp]),
        "fvh_input_number": (C.c_int, [vp, C.c_char_p, C.POINTER(C.c_double)]),
        "fvh_input_string": (C.c_int, [vp, C.c_char_p, C.c_char_p, C.c_size_t]),
        "fvh_input_params": (C.c_int, [vp, C.POINTER(Params), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int64)]),
        "fvh_input_mesh": (C.c_int, [vp, C.POINTER(vp)]),
        "fvh_input_initial_state": (C.c_int, [vp, vp, C.POINTER(Params), C.c_double, _dp]),
        "fvh_solver_autotune": (C.c_int, [vp, C.POINTER(StateView), C.c_int32,
                                          C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                          C.POINTER(C.c_int32), C.POINTER(C.c_double), vp]),
        "fvh_evaluate_time_step_noalloc": (C.c_int, [C.POINTER(MeshView), C.POINTER(StateView),
                                                     C.POINTER(Params), vp, vp, vp, vp]),
        "fvh_time_step_noalloc_max_cells": (C.c_int32, []),
        "fvh_host_mesh_concat": (C.c_int, [C.c_int32, C.POINTER(vp), C.POINTER(vp)]),
        "fvh_batch_create": (C.c_int, [C.POINTER(Params), C.c_int64, C.c_int64, C.c_int64,
                                       C.c_int32, C.POINTER(vp)]),
        "fvh_batch_destroy": (None, [vp]),
        "fvh_batch_assign": (C.c_int, [vp, C.c_int32, C.POINTER(vp), _dp, _dp,
                                       C.POINTER(C.c_int32), vp]),
        "fvh_batch_set_state": (C.c_int, [vp, C.c_int32, _dp, C.c_double, vp]),
        "fvh_batch_get_state": (C.c_int, [vp, C.c_int32, _dp, vp]),
        "fvh_batch_step": (C.c_int, [vp, C.c_int32, vp]),
        "fvh_batch_query": (C.c_int, [vp, _dp, C.POINTER(C.c_int32), C.POINTER(C.c_int64), vp]),
        "fvh_batch_set_shape": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int32]),
        "fvh_batch_num_problems": (C.c_int32, [vp]),
        "fvh_batch_autotune": (C.c_int, [vp, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_double), vp]),
        "fvh_batch_num_cells": (C.c_int64, [vp]),
        "fvh_batch_launches_per_step": (C.c_int32, [vp]),
        "fvh_solver_profile": (C.c_int, [vp, C.POINTER(StateView), C.c_int32, C.c_int32,
                                         C.POINTER(C.c_char_p), _dp, C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int32), vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def lib() -> C.CDLL:
    """Load (building first if needed) the native library."""
    global _LIB
    if _LIB is None:
        from . import _build
        path = _build.LIB
        if not os.path.exists(path) or os.environ.get("FLECSALE_GB300_REBUILD"):
            path = _build.build()
        L = C.CDLL(path)
        _declare(L)
        _LIB = L
    return _LIB


class FvhError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        msg = lib().fvh_status_string(code).decode()
        super().__init__(f"{what}: {msg} (fvh_status {code})" if what else msg)


def check(code: int, what: str = "") -> None:
    if code != OK:
        raise FvhError(code, what)


def _dptr(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError(f"expected a C-contiguous float64 array, got {a.dtype} "
                        f"(contiguous={a.flags.c_contiguous})")
    return a.ctypes.data_as(_dp)


def _iptr(a: np.ndarray):
    if a.dtype != np.int32 or not a.flags.c_contiguous:
        raise TypeError(f"expected a C-contiguous int32 array, got {a.dtype} "
                        f"(contiguous={a.flags.c_contiguous})")
    return a.ctypes.data_as(_ip)


def _state_planes(planes: np.ndarray, dim: int, num_cells: int, what: str,
                  writable: bool = False) -> np.ndarray:
    """The (5+dim, num_cells) FP64 planes d, v..., e, p, T, a the C ABI reads
    (and, for writable, writes) in full; anything smaller would be read or
    written past its end, so the shape is checked before the call."""
    if planes.shape != (5 + dim, num_cells):
        raise ValueError(f"{what}: state planes of shape {(5 + dim, num_cells)} expected, "
                         f"got {planes.shape}")
    if writable:
        if planes.dtype != np.float64 or not planes.flags.c_contiguous or not planes.flags.writeable:
            raise TypeError(f"{what}: a writable C-contiguous float64 array is required")
        return planes
    return np.ascontiguousarray(planes, np.float64)


def stream_handle(stream) -> C.c_void_p:
    """Accept None, an int handle or a torch.cuda.Stream."""
    if stream is None:
        return C.c_void_p(0)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


# ---------------------------------------------------------------------------
# host mesh
# ---------------------------------------------------------------------------
class HostMesh:
    """fvh_host_mesh: topology + FP64 geometry built on the host."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        self.view = MeshView()
        check(lib().fvh_host_mesh_view(self._h, C.byref(self.view)), "fvh_host_mesh_view")
        nnz = [C.c_int64(), C.c_int64(), C.c_int64()]
        check(lib().fvh_host_mesh_nnz(self._h, *[C.byref(x) for x in nnz]))
        self.nnz_faces, self.nnz_nbrs, self.nnz_vertices = (x.value for x in nnz)

    @classmethod
    def box(cls, dim: int, n: Sequence[int], lo: Sequence[float], hi: Sequence[float],
            jitter: float = 0.0, seed: int = 0) -> "HostMesh":
        h = C.c_void_p()
        nn = np.asarray(list(n) + [1] * (3 - len(n)), np.int32)
        l = np.asarray(list(lo) + [0.0] * (3 - len(lo)), np.float64)
        u = np.asarray(list(hi) + [1.0] * (3 - len(hi)), np.float64)
        check(lib().fvh_host_mesh_box(dim, _iptr(nn), _dptr(l), _dptr(u), jitter,
                                      C.c_uint64(seed), C.byref(h)), "fvh_host_mesh_box")
        return cls(h)

    @classmethod
    def from_cells(cls, dim: int, coords: np.ndarray, offsets: np.ndarray,
                   cells: np.ndarray) -> "HostMesh":
        coords = np.ascontiguousarray(coords, np.float64).reshape(-1)
        offsets = np.ascontiguousarray(offsets, np.int32)
        cells = np.ascontiguousarray(cells, np.int32)
        h = C.c_void_p()
        check(lib().fvh_host_mesh_create(dim, len(coords) // dim, _dptr(coords),
                                         len(offsets) - 1, _iptr(offsets), _iptr(cells),
                                         C.byref(h)), "fvh_host_mesh_create")
        return cls(h)

    def __del__(self):
        if getattr(self, "_h", None) and _LIB is not None:
            _LIB.fvh_host_mesh_destroy(self._h)
            self._h = None

    @property
    def dim(self) -> int:
        return self.view.dim

    @property
    def num_cells(self) -> int:
        return self.view.num_cells

    @property
    def num_faces(self) -> int:
        return self.view.num_faces

    @property
    def num_vertices(self) -> int:
        return self.view.num_vertices

    def _view(self, ptr, n, ctype) -> np.ndarray:
        # the ctypes array is the numpy base and holds a reference to the mesh,
        # so views outlive neither the arrays nor the mesh
        addr = C.cast(ptr, C.c_void_p).value
        if not addr:  # an empty list (a one-cell mesh has no neighbours)
            return np.zeros(0, dtype=np.dtype(ctype))
        buf = (ctype * max(n, 1)).from_address(addr)
        buf._owner = self
        return np.ctypeslib.as_array(buf)[:n]

    def _i(self, ptr, n) -> np.ndarray:
        return self._view(ptr, n, C.c_int32)

    def _d(self, ptr, n) -> np.ndarray:
        return self._view(ptr, n, C.c_double)

    def arrays(self) -> dict:
        """numpy views (no copies) of every mesh array."""
        v, D = self.view, self.dim
        nc, nf, nv = self.num_cells, self.num_faces, self.num_vertices
        return {
            "face_cells": self._i(v.face_cells, 2 * nf).reshape(nf, 2),
            "cell_face_offsets": self._i(v.cell_face_offsets, nc + 1),
            "cell_faces": self._i(v.cell_faces, self.nnz_faces),
            "cell_nbr_offsets": self._i(v.cell_nbr_offsets, nc + 1),
            "cell_nbrs": self._i(v.cell_nbrs, self.nnz_nbrs),
            "cell_vertex_offsets": self._i(v.cell_vertex_offsets, nc + 1),
            "cell_vertices": self._i(v.cell_vertices, self.nnz_vertices),
            "cell_centroid": np.stack([self._d(v.cell_centroid[d], nc) for d in range(D)]),
            "cell_volume": self._d(v.cell_volume, nc),
            "face_centroid": np.stack([self._d(v.face_centroid[d], nf) for d in range(D)]),
            "face_normal": np.stack([self._d(v.face_normal[d], nf) for d in range(D)]),
            "face_area": self._d(v.face_area, nf),
            "vertex_coord": np.stack([self._d(v.vertex_coord[d], nv) for d in range(D)]),
        }


def initial_state(kind: str, mesh: HostMesh, params: Params, seed: int = 0) -> np.ndarray:
    """(5+dim, num_cells) FP64 planes d, v..., e, p, T, a."""
    out = np.empty((5 + mesh.dim, mesh.num_cells), np.float64)
    check(lib().fvh_host_initial_state(PROBLEM[kind], mesh._h, C.byref(params),
                                       C.c_uint64(seed), _dptr(out)), "fvh_host_initial_state")
    return out


def host_state_view(planes: np.ndarray, dim: int) -> StateView:
    """StateView of host planes in the order d, v..., e, p, T, a."""
    s = StateView()
    s.density = _dptr(planes[0])
    for d in range(dim):
        s.velocity[d] = _dptr(planes[1 + d])
    s.internal_energy = _dptr(planes[1 + dim])
    s.pressure = _dptr(planes[2 + dim])
    s.temperature = _dptr(planes[3 + dim])
    s.sound_speed = _dptr(planes[4 + dim])
    return s


def gradient_view_from(buf: np.ndarray, dim: int, ptr_of=_dptr) -> GradientView:
    """GradientView over buf of shape ((dim+4)*dim, nc): rows ordered
    d[0..dim), v[0][0..dim), ..., v[dim-1][..], e[..], p[..], a[..]."""
    g = GradientView()
    r = 0
    for i in range(dim):
        g.density[i] = ptr_of(buf[r]); r += 1
    for d in range(dim):
        for i in range(dim):
            g.velocity[d][i] = ptr_of(buf[r]); r += 1
    for name in ("internal_energy", "pressure", "sound_speed"):
        arr = getattr(g, name)
        for i in range(dim):
            arr[i] = ptr_of(buf[r]); r += 1
    return g


def flux_view_from(buf: np.ndarray, dim: int, ptr_of=_dptr) -> FluxView:
    """FluxView over buf of shape (dim+2, nf): mass, momentum..., energy."""
    f = FluxView()
    f.mass = ptr_of(buf[0])
    for i in range(dim):
        f.momentum[i] = ptr_of(buf[1 + i])
    f.energy = ptr_of(buf[1 + dim])
    return f


# ---------------------------------------------------------------------------
# device objects
# ---------------------------------------------------------------------------
class DeviceMesh:
    def __init__(self, host: HostMesh):
        self._h = C.c_void_p()
        check(lib().fvh_device_mesh_create(host._h, C.byref(self._h)), "fvh_device_mesh_create")
        self.view = lib().fvh_device_mesh_view(self._h).contents
        self.dim, self.num_cells, self.num_faces = host.dim, host.num_cells, host.num_faces

    def close(self):
        if self._h and _LIB is not None:
            _LIB.fvh_device_mesh_destroy(self._h)
            self._h = None

    __del__ = close


class DeviceState:
    def __init__(self, dim: int, num_cells: int):
        self._h = C.c_void_p()
        check(lib().fvh_device_state_create(dim, num_cells, C.byref(self._h)),
              "fvh_device_state_create")
        self.view = lib().fvh_device_state_view(self._h).contents
        self.dim, self.num_cells = dim, num_cells

    def upload(self, planes: np.ndarray, stream=None) -> None:
        planes = _state_planes(np.asarray(planes), self.dim, self.num_cells, "upload")
        check(lib().fvh_state_upload(C.byref(self.view), self.dim, self.num_cells,
                                     _dptr(planes), stream_handle(stream)), "fvh_state_upload")

    def download(self, stream=None) -> np.ndarray:
        out = np.empty((5 + self.dim, self.num_cells), np.float64)
        check(lib().fvh_state_download(C.byref(self.view), self.dim, self.num_cells,
                                       _dptr(out), stream_handle(stream)), "fvh_state_download")
        return out

    def close(self):
        if self._h and _LIB is not None:
            _LIB.fvh_device_state_destroy(self._h)
            self._h = None

    __del__ = close


class Solver:
    """fvh_solver: work buffers + the time loop of apps/hydro/driver.h:317-413."""

    def __init__(self, mesh: DeviceMesh, params: Params):
        self.mesh, self.params = mesh, params
        self._h = C.c_void_p()
        check(lib().fvh_solver_create(C.byref(mesh.view), C.byref(params), C.byref(self._h)),
              "fvh_solver_create")

    def step(self, state: DeviceState, stream=None) -> None:
        check(lib().fvh_solver_step(self._h, C.byref(state.view), stream_handle(stream)),
              "fvh_solver_step")

    def run(self, state: DeviceState, nsteps: int, stop_at_final_time: bool = False,
            check_every: int = 1, stream=None) -> int:
        done = C.c_int64()
        check(lib().fvh_solver_run(self._h, C.byref(state.view), nsteps,
                                   1 if stop_at_final_time else 0, check_every,
                                   C.byref(done), stream_handle(stream)), "fvh_solver_run")
        return done.value

    def status(self, stream=None) -> tuple[int, float, int]:
        t, cell = C.c_double(), C.c_int64()
        code = lib().fvh_solver_check(self._h, stream_handle(stream), C.byref(t), C.byref(cell))
        return code, t.value, cell.value

    def soln_time(self, stream=None) -> float:
        return self.status(stream)[1]

    def reset(self, t: float = 0.0, stream=None) -> None:
        check(lib().fvh_solver_reset(self._h, t, stream_handle(stream)), "fvh_solver_reset")

    def advance_host(self, state: DeviceState, planes: np.ndarray, nsteps: int, t: float,
                     stream=None) -> float:
        _state_planes(planes, state.dim, state.num_cells, "advance_host", writable=True)
        tt = C.c_double(t)
        check(lib().fvh_solver_advance_host(self._h, C.byref(state.view), _dptr(planes),
                                            nsteps, C.byref(tt), stream_handle(stream)),
              "fvh_solver_advance_host")
        return tt.value

    def launches_per_step(self) -> int:
        return lib().fvh_solver_launches_per_step(self._h)

    def set_shape(self, block: int, cells_per_thread: int, schedule: int = 0) -> None:
        check(lib().fvh_solver_set_shape(self._h, block, cells_per_thread, schedule),
              "fvh_solver_set_shape")

    def autotune(self, state: DeviceState, trial_steps: int = 5, stream=None) -> dict:
        """Times each launch shape on a scratch copy of `state`; keeps the fastest."""
        blk, cpt, sch, ms = C.c_int32(), C.c_int32(), C.c_int32(), C.c_double()
        check(lib().fvh_solver_autotune(self._h, C.byref(state.view), trial_steps, C.byref(blk),
                                        C.byref(cpt), C.byref(sch), C.byref(ms),
                                        stream_handle(stream)), "fvh_solver_autotune")
        return {"block": blk.value, "cells_per_thread": cpt.value, "schedule": sch.value,
                "ms_per_step": ms.value}

    def profile(self, state: DeviceState, nsteps: int, stream=None) -> dict:
        """{kernel name: (mean ms per launch, launches per step)} over nsteps steps
        launched as a run launches them."""
        mx = 16
        names = (C.c_char_p * mx)()
        ms = np.zeros(mx)
        per = (C.c_int32 * mx)()
        nk = C.c_int32()
        check(lib().fvh_solver_profile(self._h, C.byref(state.view), nsteps, mx, names, _dptr(ms),
                                       per, C.byref(nk), stream_handle(stream)), "fvh_solver_profile")
        return {names[k].decode(): (float(ms[k]), per[k] / nsteps) for k in range(nk.value)}

    def launches_per_run(self, nsteps: int) -> int:
        return lib().fvh_solver_launches_per_run(self._h, nsteps)

    @property
    def d_soln_time(self) -> int:
        return lib().fvh_solver_soln_time(self._h)

    @property
    def d_dt(self) -> int:
        return lib().fvh_solver_dt(self._h)

    @property
    def d_status(self) -> int:
        return lib().fvh_solver_status(self._h)

    @property
    def gradients(self) -> GradientView:
        return lib().fvh_solver_gradients(self._h).contents

    @property
    def fluxes(self) -> FluxView:
        return lib().fvh_solver_fluxes(self._h).contents

    def close(self):
        if self._h and _LIB is not None:
            _LIB.fvh_solver_destroy(self._h)
            self._h = None

    __del__ = close


class Batch:
    """fvh_batch: independent meshes advanced together (mixed precision)."""

    def __init__(self, params: Params, max_cells: int, max_faces: int, max_vertices: int,
                 max_problems: int):
        self.params = params
        self.dim = params.dim
        self._h = C.c_void_p()
        check(lib().fvh_batch_create(C.byref(params), max_cells, max_faces, max_vertices,
                                     max_problems, C.byref(self._h)), "fvh_batch_create")
        self.meshes: list = []

    @classmethod
    def for_meshes(cls, params: Params, meshes, slack: float = 1.0, max_problems=None):
        nc = sum(m.num_cells for m in meshes)
        nf = sum(m.num_faces for m in meshes)
        nv = sum(m.num_vertices for m in meshes)
        return cls(params, int(nc * slack) + 1, int(nf * slack) + 1, int(nv * slack) + 1,
                   max_problems or len(meshes))

    def assign(self, meshes, cfl, final_time, keep=None, stream=None) -> None:
        n = len(meshes)
        arr = (C.c_void_p * n)(*[m._h for m in meshes])
        cf = np.ascontiguousarray(np.broadcast_to(np.asarray(cfl, np.float64), (n,)))
        tf = np.ascontiguousarray(np.broadcast_to(np.asarray(final_time, np.float64), (n,)))
        kp = None if keep is None else (C.c_int32 * n)(*keep)
        check(lib().fvh_batch_assign(self._h, n, arr, _dptr(cf), _dptr(tf), kp,
                                     stream_handle(stream)), "fvh_batch_assign")
        self.meshes = list(meshes)

    def set_state(self, k: int, planes: np.ndarray, t: float = 0.0, stream=None) -> None:
        if not 0 <= k < len(self.meshes):
            raise IndexError(f"set_state: problem {k} of {len(self.meshes)}")
        planes = _state_planes(np.asarray(planes)[:5 + self.dim], self.dim,
                               self.meshes[k].num_cells, "set_state")
        check(lib().fvh_batch_set_state(self._h, k, _dptr(planes), t, stream_handle(stream)),
              "fvh_batch_set_state")

    def get_state(self, k: int, stream=None) -> np.ndarray:
        out = np.empty((5 + self.dim, self.meshes[k].num_cells), np.float64)
        check(lib().fvh_batch_get_state(self._h, k, _dptr(out), stream_handle(stream)),
              "fvh_batch_get_state")
        return out

    def step(self, nsteps: int = 1, stream=None) -> None:
        check(lib().fvh_batch_step(self._h, nsteps, stream_handle(stream)), "fvh_batch_step")

    def query(self, stream=None):
        n = lib().fvh_batch_num_problems(self._h)
        t = np.zeros(n)
        codes = (C.c_int32 * n)()
        bad = (C.c_int64 * n)()
        rc = lib().fvh_batch_query(self._h, _dptr(t), codes, bad, stream_handle(stream))
        # a failed problem (negative state, infinite dt) is reported in its own
        # code; only argument and CUDA errors fail the query itself
        if rc not in (OK, ERR_NEGATIVE_STATE, ERR_INFINITE_DT):
            check(rc, "fvh_batch_query")
        return t, np.array(codes[:], np.int32), np.array(bad[:], np.int64)

    def set_shape(self, block: int, cells_per_thread: int, schedule: int = 0) -> None:
        check(lib().fvh_batch_set_shape(self._h, block, cells_per_thread, schedule),
              "fvh_batch_set_shape")

    def autotune(self, trial_steps: int = 3, use_cache: bool = True, stream=None) -> dict:
        blk, cpt, sch, ms = C.c_int32(), C.c_int32(), C.c_int32(), C.c_double()
        check(lib().fvh_batch_autotune(self._h, trial_steps, 1 if use_cache else 0, C.byref(blk),
                                       C.byref(cpt), C.byref(sch), C.byref(ms),
                                       stream_handle(stream)), "fvh_batch_autotune")
        return {"block": blk.value, "cells_per_thread": cpt.value, "schedule": sch.value,
                "ms_per_step": ms.value}

    @property
    def num_cells(self) -> int:
        return lib().fvh_batch_num_cells(self._h)

    def launches_per_step(self) -> int:
        return lib().fvh_batch_launches_per_step(self._h)

    def close(self):
        if self._h and _LIB is not None:
            _LIB.fvh_batch_destroy(self._h)
            self._h = None

    __del__ = close


def _declare_io(L: C.CDLL) -> None:
    vp = C.c_void_p
    for name, res, args in [
        ("fvh_host_mesh_read_exodus", C.c_int, [C.c_char_p, C.POINTER(vp)]),
        ("fvh_dump_write", C.c_int, [C.c_char_p, vp, _dp, C.c_double, C.c_int64]),
        ("fvh_host_state_from_dvp", C.c_int, [C.c_int32, C.c_int32, C.c_double, C.c_double,
                                               _dp, _dp, _dp, _dp]),
        ("fvh_dump_read", C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                    _dp, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    ]:
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args


def read_exodus(path: str) -> HostMesh:
    """Mesh from an Exodus II file (netCDF classic / 64-bit offset)."""
    _declare_io(lib())
    h = C.c_void_p()
    check(lib().fvh_host_mesh_read_exodus(path.encode(), C.byref(h)), f"read_exodus({path})")
    return HostMesh(h)


def write_dump(path: str, mesh: HostMesh, planes: np.ndarray, soln_time: float,
               iterations: int) -> None:
    """Regression dump in the reference's format (apps/hydro/tasks.h:771-849)."""
    _declare_io(lib())
    planes = _state_planes(np.asarray(planes)[:5 + mesh.dim], mesh.dim, mesh.num_cells,
                           "write_dump")
    check(lib().fvh_dump_write(path.encode(), mesh._h, _dptr(planes), soln_time, iterations),
          "fvh_dump_write")


def read_dump(path: str, dim: int, num_cells: int, gamma: float = 1.4,
              cv: float = 1.0) -> tuple:
    """(state planes, solution time, iterations) from a regression dump
    (fvh_dump_read): resumes a run from the text the reference's dump task
    and write_dump produce."""
    _declare_io(lib())
    out = np.empty((5 + dim, num_cells), np.float64)
    t, n = C.c_double(), C.c_int64()
    check(lib().fvh_dump_read(path.encode(), dim, num_cells, gamma, cv, _dptr(out), C.byref(t),
                              C.byref(n)), f"read_dump({path})")
    return out, t.value, n.value


def state_from_dvp(dim: int, density, velocity, pressure, gamma: float = 1.4,
                   cv: float = 1.0) -> np.ndarray:
    """State planes (d, v..., e, p, T, a) from density, velocity [dim][n] and pressure."""
    _declare_io(lib())
    d = np.ascontiguousarray(density, np.float64)
    v = np.ascontiguousarray(velocity, np.float64).reshape(dim, -1)
    p = np.ascontiguousarray(pressure, np.float64)
    out = np.empty((5 + dim, d.size), np.float64)
    check(lib().fvh_host_state_from_dvp(dim, d.size, gamma, cv, _dptr(d), _dptr(v), _dptr(p),
                                        _dptr(out)), "fvh_host_state_from_dvp")
    return out


def _declare_batch_device(L: C.CDLL) -> None:
    fn = L.fvh_batch_assign_device
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), _dp, _dp, C.POINTER(C.c_int32),
                   C.c_void_p]


def batch_assign_device(batch: "Batch", dmeshes, cfl, final_time, keep=None, stream=None) -> None:
    """fvh_batch_assign_device: problems already resident in device memory
    (DeviceMesh) are concatenated on the device."""
    _declare_batch_device(lib())
    n = len(dmeshes)
    arr = (C.c_void_p * n)(*[m._h for m in dmeshes])
    cf = np.ascontiguousarray(np.broadcast_to(np.asarray(cfl, np.float64), (n,)))
    tf = np.ascontiguousarray(np.broadcast_to(np.asarray(final_time, np.float64), (n,)))
    kp = None if keep is None else (C.c_int32 * n)(*keep)
    check(lib().fvh_batch_assign_device(batch._h, n, arr, _dptr(cf), _dptr(tf), kp,
                                        stream_handle(stream)), "fvh_batch_assign_device")
    batch.meshes = list(dmeshes)


class Input:
    """An apps/hydro input file (the Lua "hydro" table, inputs.h:100-135)."""

    def __init__(self, path: str | None = None, text: str | None = None):
        self._h = C.c_void_p()
        err = C.create_string_buffer(512)
        if path is not None:
            code = lib().fvh_input_load(path.encode(), err, 512, C.byref(self._h))
        else:
            code = lib().fvh_input_load_string(text.encode(), err, 512, C.byref(self._h))
        if code != 0:
            # the message may quote bytes of the file that are not UTF-8
            raise FvhError(code, err.value.decode(errors="replace") or "fvh_input_load")

    def number(self, path: str) -> float:
        v = C.c_double()
        check(lib().fvh_input_number(self._h, path.encode(), C.byref(v)), path)
        return v.value

    def string(self, path: str) -> str:
        buf = C.create_string_buffer(4096)
        check(lib().fvh_input_string(self._h, path.encode(), buf, 4096), path)
        return buf.value.decode(errors="replace")

    def params(self, dim: int, **kw) -> tuple:
        """(Params, max_steps, output_freq): reference defaults for dim, then the file."""
        p = make_params(dim, **kw)
        ms, of = C.c_int64(-1), C.c_int64(-1)
        check(lib().fvh_input_params(self._h, C.byref(p), C.byref(ms), C.byref(of)),
              "fvh_input_params")
        return p, ms.value, of.value

    def mesh(self) -> "HostMesh":
        h = C.c_void_p()
        check(lib().fvh_input_mesh(self._h, C.byref(h)), "fvh_input_mesh")
        return HostMesh(h)

    def initial_state(self, mesh: "HostMesh", params: Params, t: float = 0.0) -> np.ndarray:
        out = np.empty((5 + mesh.dim, mesh.num_cells), np.float64)
        check(lib().fvh_input_initial_state(self._h, mesh._h, C.byref(params), t, _dptr(out)),
              "fvh_input_initial_state")
        return out

    def close(self):
        if self._h and _LIB is not None:
            _LIB.fvh_input_destroy(self._h)
            self._h = None

    __del__ = close


def driver_path() -> str:
    """The flecsale_hydro command-line driver built beside the library."""
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "flecsale_hydro")
