"""Properties the oracle must have whatever the reference's unpinned mesh
orders are (CPU only): free-stream preservation on jittered and unstructured
meshes, direction invariance and dimension independence of a 1D problem, and
convergence to the exact Riemann solution on jittered meshes.  The GPU FP64
path is bitwise equal to the oracle, so these hold for it as well."""
import numpy as np
import pytest

import flecsale_gb300.hydro as H
from tests import _util as U
from tests.test_exact_riemann import GAMMA, SOD_L, SOD_R, exact_riemann

MESHES = {
    "quads_jittered": lambda: H.HostMesh.box(2, (24, 20), [0, 0], [1, 1], 0.2, 5),
    "quad_tri_mix": lambda: U.tri_mesh((20, 16), split_every=3),
    "triangles": lambda: U.tri_mesh((16, 14)),
    "hexes_jittered": lambda: H.HostMesh.box(3, (8, 7, 6), [0, 0, 0], [1, 1, 1], 0.15, 6),
    "tetrahedra": lambda: U.tet_mesh((4, 4, 3)),
}


def _uniform(mesh, velocity, p):
    n = mesh.num_cells
    v = np.array(velocity[:mesh.dim], np.float64)[:, None] * np.ones((mesh.dim, n))
    return H.state_from_dvp(mesh.dim, np.full(n, 1.3), v, np.full(n, 0.7), p.gamma, p.cv)


@pytest.mark.parametrize("name", sorted(MESHES))
@pytest.mark.parametrize("flux", ["hllc", "hlle", "rusanov"])
def test_free_stream_is_preserved(fvh, oracle_lib, name, flux):
    """A uniform flow through outflow boundaries, and a gas at rest between
    walls, stay uniform to round-off after second-order steps: each cell's
    face normals times areas must close (sum to zero) for that to hold."""
    mesh = MESHES[name]()
    for boundary, vel in (("outflow", (0.31, -0.23, 0.17)), ("wall", (0.0, 0.0, 0.0))):
        p = H.make_params(mesh.dim, flux=flux, boundary=boundary, swap=False, cfl=0.4)
        s0 = _uniform(mesh, vel, p)
        s = s0.copy()
        st, t, n = U.oracle_run(oracle_lib, mesh, s, p, 6)
        assert st == 0 and n == 6 and t > 0
        scale = np.abs(s0).max(axis=1, keepdims=True)
        assert np.abs(s - s0).max() <= 1e-12 * scale.max(), (boundary, np.abs(s - s0).max(axis=1))


def _sod_along(axis, dim, n=100, m=3):
    """Sod along one axis of an n x m (x m) box with square cells."""
    shape = [m] * dim
    shape[axis] = n
    hi = [m / n] * dim
    hi[axis] = 1.0
    mesh = H.HostMesh.box(dim, shape, [0] * dim, hi)
    p = H.make_params(dim, flux="hllc", order=1, cfl=0.5, final_time=0.2)
    x = mesh.arrays()["cell_centroid"][axis]
    left = x < 0.5
    s = H.state_from_dvp(dim, np.where(left, 1.0, 0.125), np.zeros((dim, mesh.num_cells)),
                         np.where(left, 1.0, 0.1), p.gamma, p.cv)
    return mesh, p, s, x


def test_sod_is_the_same_along_every_axis_and_in_2d_and_3d(fvh, oracle_lib):
    """First-order HLLC Sod along x, y and z of a 3D box and along x and y of
    a 2D box: the same density profile (to 1e-12), within first-order distance
    of the exact solution."""
    profiles = []
    for dim, axis in ((2, 0), (2, 1), (3, 0), (3, 1), (3, 2)):
        mesh, p, s, x = _sod_along(axis, dim)
        st, t, _ = U.oracle_run(oracle_lib, mesh, s, p, 100000, stop_at_final=True)
        assert st == 0 and abs(t - 0.2) <= 1e-14
        order = np.argsort(x, kind="stable")
        prof = s[0][order].reshape(100, -1)
        assert np.abs(prof - prof[:, :1]).max() <= 1e-12  # every transverse line the same
        profiles.append(prof[:, 0])
        vt = [s[1 + d] for d in range(dim) if d != axis]
        assert max(np.abs(v).max() for v in vt) <= 1e-12  # no transverse velocity
        xs = np.sort(x)[::len(x) // 100][:100]
        exact = exact_riemann(SOD_L, SOD_R, GAMMA, (xs - 0.5) / t)[0]
        assert np.abs(prof[:, 0] - exact).mean() <= 0.021
    for q in profiles[1:]:
        assert np.abs(q - profiles[0]).max() <= 1e-12


def test_sod_on_jittered_meshes_converges(fvh, oracle_lib):
    """Sod on quads whose interior nodes are jittered by +-0.2h: the L1
    density error against the exact solution is within 1.3x of the uniform
    mesh's and falls by at least 1.3x per mesh doubling (first-order HLLC)."""
    err = {}
    for jit in (0.0, 0.2):
        for n in (100, 200):
            mesh = H.HostMesh.box(2, (n, n // 10), [0, 0], [1, 0.1], jit, 11)
            p = H.make_params(2, flux="hllc", order=1, cfl=0.5, final_time=0.2)
            s = H.initial_state("sod", mesh, p)
            st, t, _ = U.oracle_run(oracle_lib, mesh, s, p, 100000, stop_at_final=True)
            assert st == 0
            a = mesh.arrays()
            exact = exact_riemann(SOD_L, SOD_R, GAMMA, (a["cell_centroid"][0] - 0.5) / t)[0]
            vol = a["cell_volume"]
            err[jit, n] = float((np.abs(s[0] - exact) * vol).sum() / vol.sum())
    assert err[0.2, 100] <= 1.3 * err[0.0, 100], err
    assert err[0.2, 100] / err[0.2, 200] >= 1.3, err


@pytest.mark.parametrize("flux", ["hllc", "hlle", "rusanov"])
def test_four_quadrant_keeps_its_diagonal_symmetry(fvh, oracle_lib, flux):
    """The four-quadrant problem is symmetric about x = y (NW and SE swap
    under x <-> y with u <-> v): on an unjittered 64^2 mesh, 40 second-order
    steps keep rho(x, y) = rho(y, x) and u(x, y) = v(y, x) to rounding
    (measured 1.4e-13 and 1.1e-12 with HLLC), so x and y take the same paths
    through the gradients, the limiter and the fluxes."""
    n = 64
    mesh = H.HostMesh.box(2, (n, n), [0, 0], [1, 1])
    p = H.make_params(2, flux=flux, cfl=0.4, boundary="outflow", swap=False)
    s = H.initial_state("four_quadrant", mesh, p)
    st, t, _ = U.oracle_run(oracle_lib, mesh, s, p, 40)
    assert st == 0 and t > 0
    d, u, v, e = (s[k].reshape(n, n) for k in (0, 1, 2, 3))  # [y, x]
    assert np.abs(d - d.T).max() <= 1e-11
    assert np.abs(u - v.T).max() <= 1e-10 and np.abs(e - e.T).max() <= 1e-10
    assert np.abs(d - d[::-1]).max() > 0.1  # the solution is not trivially symmetric otherwise


@pytest.mark.parametrize("flux", ["rusanov", "hllc", "hlle"])
@pytest.mark.parametrize("boundary", ["wall", "outflow"])
def test_inner_cube_keeps_its_axis_symmetry(fvh, oracle_lib, flux, boundary):
    """The 3D inner-cube problem is symmetric under any exchange of axes: on
    an unjittered 24^3 hex mesh, 20 second-order steps keep the density and
    the velocity components permutation-symmetric to rounding (measured
    <= 8e-15), so the three directions take the same paths through the 3D
    gradients, limiter and fluxes."""
    n = 24
    mesh = H.HostMesh.box(3, (n, n, n), [0] * 3, [1] * 3)
    p = H.make_params(3, flux=flux, cfl=0.3, boundary=boundary, swap=False)
    s = H.initial_state("inner_cube", mesh, p)
    st, _, _ = U.oracle_run(oracle_lib, mesh, s, p, 20)
    assert st == 0
    d = s[0].reshape(n, n, n)  # [z, y, x]
    vx, vy, vz = (s[1 + k].reshape(n, n, n) for k in range(3))
    xy, xz = (0, 2, 1), (2, 1, 0)
    assert np.abs(d - d.transpose(xy)).max() <= 1e-13
    assert np.abs(d - d.transpose(xz)).max() <= 1e-13
    assert np.abs(vx - vy.transpose(xy)).max() <= 1e-13
    assert np.abs(vx - vz.transpose(xz)).max() <= 1e-13
    assert np.abs(d - d[::-1]).max() > 0.1  # the shock has moved: a non-trivial state
