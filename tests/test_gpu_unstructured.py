"""The GPU path on cell shapes other than the box generator's quads and hexes:
triangles, a quad/triangle mix and tetrahedra (Exodus TRI3/QUAD4 polygons and
TETRA4), with more vertex neighbours than the box cells have.  FP64 runs are
bitwise equal to the oracle; the mixed form is within the 1e-4 L1 bar."""
import numpy as np
import pytest

import flecsale_gb300.hydro as H
from tests import _util as U

pytestmark = pytest.mark.gpu


def _tri_mesh(n=(30, 22), split_every=1, seed=3):
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


def _tet_mesh(n=(6, 5, 5), seed=2):
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


def _run(mesh, p, state, nsteps):
    dm, ds = H.DeviceMesh(mesh), H.DeviceState(mesh.dim, mesh.num_cells)
    s = H.Solver(dm, p)
    ds.upload(state)
    s.reset(0.0)
    assert s.run(ds, nsteps) == nsteps
    code, t, _ = s.status()
    assert code == 0
    return ds.download(), t


MESHES = {
    "triangles": lambda: _tri_mesh(),
    "quad_tri_mix": lambda: _tri_mesh(split_every=3),
    "tetrahedra": lambda: _tet_mesh(),
}


@pytest.mark.parametrize("name", list(MESHES))
def test_fp64_bitwise_and_mixed_close(cuda, name):
    mesh = MESHES[name]()
    dim = mesh.dim
    kw = dict(flux="hllc", cfl=0.4 if dim == 2 else 0.3, boundary="outflow")
    p = H.make_params(dim, **kw)
    s0 = H.initial_state("four_quadrant" if dim == 2 else "inner_cube", mesh, p, seed=3)
    nsteps = 12
    gpu, t_gpu = _run(mesh, p, s0, nsteps)
    ref = s0.copy()
    st, t, n = U.oracle_run(__import__("oracle").load(), mesh, ref, p, nsteps)
    assert st == 0 and n == nsteps and t == t_gpu
    assert np.array_equal(gpu, ref)
    mix, t_mix = _run(mesh, H.make_params(dim, precision="mixed", **kw), s0, nsteps)
    assert abs(t_mix - t) <= 1e-4 * t
    assert np.abs(mix[0] - ref[0]).sum() / np.abs(ref[0]).sum() <= 1e-4
    if dim == 3:  # tet vertex neighbourhoods are larger than a hex's 26
        assert mesh.nnz_nbrs / mesh.num_cells > 26
