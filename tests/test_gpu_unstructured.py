"""The GPU path on cell shapes other than the box generator's quads and hexes:
triangles, a quad/triangle mix and tetrahedra (Exodus TRI3/QUAD4 polygons and
TETRA4), with more vertex neighbours than the box cells have.  FP64 runs are
bitwise equal to the oracle; the mixed form is within the 1e-4 L1 bar."""
import numpy as np
import pytest

import flecsale_gb300.hydro as H
from tests import _util as U

pytestmark = pytest.mark.gpu


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
    "triangles": lambda: U.tri_mesh(),
    "quad_tri_mix": lambda: U.tri_mesh(split_every=3),
    "tetrahedra": lambda: U.tet_mesh(),
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
