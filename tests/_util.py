"""Shared helpers for the tests: oracle calls on host arrays, golden meshes,
and device views over torch tensors (torch is only device-memory plumbing)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

import flecsale_gb300.hydro as H

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# the reference checkout named by FLECSALE_REFERENCE, for the tests that also
# check against it; they skip when it is unset
REFERENCE = os.environ.get("FLECSALE_REFERENCE", "")


# ---------------------------------------------------------------------------
# golden meshes
# ---------------------------------------------------------------------------
def golden_2d():
    """32x32 mesh of apps/hydro/2d rebuilt from its regression dump: vertex ids
    and coordinates as listed; each cell's corners found from its centroid,
    listed counter-clockwise from the (+x,+y) corner like cell 0 in the dump."""
    z = np.load(os.path.join(GOLDEN, "shock_box_2d_32x32.npz"))
    vc, cc = z["vertex_coord"], z["cell_centroid"]
    h = 1.0 / 32
    key = {(int(round((x + 0.5) / h)), int(round((y + 0.5) / h))): i for i, (x, y) in enumerate(vc)}
    corners = [(1, 1), (-1, 1), (-1, -1), (1, -1)]
    cells = np.array([[key[(int(round((x + 0.5) / h + sx * 0.5)), int(round((y + 0.5) / h + sy * 0.5)))]
                       for sx, sy in corners] for x, y in cc], np.int32)
    mesh = H.HostMesh.from_cells(2, vc, np.arange(0, 4 * len(cells) + 1, 4, dtype=np.int32),
                                 cells.reshape(-1))
    return mesh, z


def golden_3d():
    """20^3 HEX8 mesh of apps/hydro/3d (data/meshes/sedov_20x20x20.g)."""
    z = np.load(os.path.join(GOLDEN, "shock_box_3d_20x20x20.npz"))
    cn = z["exodus_connect"]
    mesh = H.HostMesh.from_cells(3, z["exodus_coord"], np.arange(0, 8 * len(cn) + 1, 8, dtype=np.int32),
                                 cn.reshape(-1))
    return mesh, z


def two_rank_dumps():
    """Per-rank dumps of apps/hydro/2d run on two ranks (544 cells each,
    owned and ghost), from shock_box_2d_32x32_2procs.npz."""
    return np.load(os.path.join(GOLDEN, "shock_box_2d_32x32_2procs.npz"))


def two_rank_max_diff(cols: np.ndarray, centroids: np.ndarray, z2) -> float:
    """Largest |difference| between single-domain dump columns (cells in the
    order of `centroids`) and every cell listed in the two rank dumps, cells
    matched by centroid (the ranks number their cells differently)."""
    key = {(round(float(x), 9), round(float(y), 9)): i for i, (x, y) in enumerate(centroids)}
    worst = 0.0
    for r in (0, 1):
        for (x, y), row in zip(z2[f"rank{r}_centroid"], z2[f"rank{r}_cells"]):
            worst = max(worst, float(np.abs(cols[key[(round(float(x), 9), round(float(y), 9))]] - row).max()))
    return worst


def dump_columns(state: np.ndarray, dim: int) -> np.ndarray:
    """Cell columns of the reference dump: density internal_energy pressure velocity..."""
    return np.stack([state[0], state[1 + dim], state[2 + dim], *[state[1 + d] for d in range(dim)]], 1)


def numdiff_ok(expected: np.ndarray, actual: np.ndarray, abs_tol: float = 1e-14) -> bool:
    """tools/numdiff.py --absolute semantics (softEquiv, numdiff.py:70-96)."""
    return bool(np.all(np.abs(actual - expected) <= abs_tol))


# ---------------------------------------------------------------------------
# unstructured meshes (Exodus TRI3/QUAD4 polygons and TETRA4 cells)
# ---------------------------------------------------------------------------
def tri_mesh(n=(30, 22), split_every=1, seed=3):
    """A jittered quad box with every split_every-th quad cut into two
    triangles (alternating diagonals)."""
    box = H.HostMesh.box(2, n, [0, 0], [1, 1], 0.2, seed)
    a = box.arrays()
    coords = a["vertex_coord"].T.copy()
    quads = a["cell_vertices"].reshape(-1, 4)
    cells, offs = [], [0]
    for k, q in enumerate(quads):
        if k % split_every == 0:
            t = ((q[0], q[1], q[2]), (q[0], q[2], q[3])) if k % 2 else \
                ((q[0], q[1], q[3]), (q[1], q[2], q[3]))
            for tri in t:
                cells += tri
                offs.append(len(cells))
        else:
            cells += list(q)
            offs.append(len(cells))
    return H.HostMesh.from_cells(2, coords, np.array(offs, np.int32), np.array(cells, np.int32))


def tet_mesh(n=(6, 5, 5), seed=2):
    """A jittered hex box with each hex cut into 6 tetrahedra around its main
    diagonal, each ordered to positive volume."""
    box = H.HostMesh.box(3, n, [0, 0, 0], [1, 1, 1], 0.15, seed)
    a = box.arrays()
    x = a["vertex_coord"].T.copy()
    hexes = a["cell_vertices"].reshape(-1, 8)
    cells = []
    for h in hexes:
        for t in ((0, 1, 2, 6), (0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 4, 5, 6), (0, 5, 1, 6)):
            v = [h[i] for i in t]
            d = np.linalg.det(np.stack([x[v[1]] - x[v[0]], x[v[2]] - x[v[0]], x[v[3]] - x[v[0]]]))
            if d < 0:
                v[1], v[2] = v[2], v[1]
            cells += v
    return H.HostMesh.from_cells(3, x, np.arange(0, len(cells) + 1, 4, dtype=np.int32),
                                 np.array(cells, np.int32))


# ---------------------------------------------------------------------------
# oracle calls on host arrays
# ---------------------------------------------------------------------------
def grad_rows(dim: int) -> int:
    return (dim + 4) * dim


def oracle_gradients(O, mesh, state, params):
    g = np.zeros((grad_rows(mesh.dim), mesh.num_cells))
    O.oracle_evaluate_gradients(C.byref(mesh.view), C.byref(H.host_state_view(state, mesh.dim)),
                                C.byref(H.gradient_view_from(g, mesh.dim)), C.byref(params))
    return g


def oracle_fluxes(O, mesh, state, grads, params):
    f = np.zeros((mesh.dim + 2, mesh.num_faces))
    O.oracle_evaluate_fluxes(C.byref(mesh.view), C.byref(H.host_state_view(state, mesh.dim)),
                             C.byref(H.gradient_view_from(grads, mesh.dim)),
                             C.byref(H.flux_view_from(f, mesh.dim)), C.byref(params))
    return f


def oracle_time_step(O, mesh, state, params, t=0.0):
    dt = C.c_double()
    st = O.oracle_evaluate_time_step(C.byref(mesh.view), C.byref(H.host_state_view(state, mesh.dim)),
                                     C.byref(params), t, C.byref(dt))
    return st, dt.value


def oracle_update(O, mesh, state, flux, params, dt, factor, t=0.0):
    """Updates state in place; returns (status, new time, bad cell)."""
    tt, bad = C.c_double(t), C.c_int64(-1)
    st = O.oracle_apply_update(C.byref(mesh.view), C.byref(params), dt, factor,
                               C.byref(H.flux_view_from(flux, mesh.dim)),
                               C.byref(H.host_state_view(state, mesh.dim)), C.byref(tt), C.byref(bad))
    return st, tt.value, bad.value


def oracle_run(O, mesh, state, params, nsteps, stop_at_final=False, t=0.0):
    tt, n, bad = C.c_double(t), C.c_int64(), C.c_int64(-1)
    st = O.oracle_run(C.byref(mesh.view), C.byref(params), C.byref(H.host_state_view(state, mesh.dim)),
                      nsteps, 1 if stop_at_final else 0, C.byref(tt), C.byref(n), C.byref(bad))
    return st, tt.value, n.value


# ---------------------------------------------------------------------------
# device views over torch tensors
# ---------------------------------------------------------------------------
def _row_ptrs(t):
    base, stride = t.data_ptr(), t.stride(0) * t.element_size()
    return [C.cast(C.c_void_p(base + r * stride), C.POINTER(C.c_double)) for r in range(t.shape[0])]


def device_state_view(t, dim: int) -> H.StateView:
    p = _row_ptrs(t)
    s = H.StateView()
    s.density = p[0]
    for d in range(dim):
        s.velocity[d] = p[1 + d]
    s.internal_energy, s.pressure, s.temperature, s.sound_speed = p[1 + dim], p[2 + dim], p[3 + dim], p[4 + dim]
    return s


def device_gradient_view(t, dim: int) -> H.GradientView:
    p = _row_ptrs(t)
    return H.gradient_view_from(list(range(t.shape[0])), dim, ptr_of=lambda r: p[r])


def device_flux_view(t, dim: int) -> H.FluxView:
    p = _row_ptrs(t)
    return H.flux_view_from(list(range(t.shape[0])), dim, ptr_of=lambda r: p[r])
