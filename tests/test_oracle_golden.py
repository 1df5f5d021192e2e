"""Pin the oracle to the reference's own regression goldens and known answers.

- apps/hydro/2d regression (2d/CMakeLists.txt:23-47): 32x32 shock box, 20 steps,
  compared with shock_box_2d-solution_rank000000.txt.1procs.std using the
  reference's numdiff semantics, absolute 1e-14 (cmake/regression.cmake:19).
- apps/hydro/3d regression (3d/CMakeLists.txt:23-62): 20^3 hexes, 12 steps,
  uniform state stays uniform.
- ideal gas known answers (flecsale/eos/test/ideal_gas.cc:40-79).
"""
import ctypes as C

import numpy as np
import pytest

from tests import _util as U


def test_golden_2d_shock_box(fvh, oracle_lib):
    mesh, z = U.golden_2d()
    p = fvh.make_params(2)  # HLLE, Barth-Jespersen, swap, gamma 1.4, CFL 1/2 (2d/inputs.cc:27-42)
    state = fvh.initial_state("shock_box", mesh, p)
    st, t, n = U.oracle_run(oracle_lib, mesh, state, p, int(z["iterations"]))
    assert st == 0 and n == 20
    assert abs(t - float(z["soln_time"])) <= 1e-14
    cols = U.dump_columns(state, 2)
    assert U.numdiff_ok(z["cells"], cols, 1e-14)
    # the run is not trivial: the shock has moved through most of the box
    assert z["cells"][:, 0].min() < 0.11 and z["cells"][:, 0].max() > 1.0


def test_golden_2d_two_rank_dumps(fvh, oracle_lib):
    """The same problem run by the reference on two ranks lists 544 cells per
    rank (owned and ghost); every one matches the single-domain oracle run
    within the reference's regression tolerance (numdiff abs 1e-14; measured
    8.4e-15, while the reference's own 1-rank and 2-rank dumps differ by up
    to 1.02e-14)."""
    mesh, z = U.golden_2d()
    z2 = U.two_rank_dumps()
    assert int(z2["iterations"]) == int(z["iterations"])
    assert float(z2["soln_time"]) == float(z["soln_time"])
    assert len(z2["rank0_cells"]) == len(z2["rank1_cells"]) == 544
    # the two ranks together list every cell
    ids = set(z2["rank0_global_id"].tolist()) | set(z2["rank1_global_id"].tolist())
    assert len(ids) == mesh.num_cells
    p = fvh.make_params(2)
    state = fvh.initial_state("shock_box", mesh, p)
    st, _, _ = U.oracle_run(oracle_lib, mesh, state, p, int(z["iterations"]))
    assert st == 0
    assert U.two_rank_max_diff(U.dump_columns(state, 2), z["cell_centroid"], z2) <= 1e-14


def test_golden_2d_needs_the_reference_quirks(fvh, oracle_lib):
    """Without the e/p gradient swap (tasks.h:429-430) or with Rusanov instead of
    HLLE (types.h:118-125) the golden is not reproduced."""
    mesh, z = U.golden_2d()
    for kw in ({"swap": False}, {"flux": "rusanov"}):
        p = fvh.make_params(2, **kw)
        state = fvh.initial_state("shock_box", mesh, p)
        U.oracle_run(oracle_lib, mesh, state, p, 20)
        assert np.abs(U.dump_columns(state, 2)[:, 0] - z["cells"][:, 0]).max() > 1e-3


def test_golden_2d_mesh_geometry(fvh):
    mesh, z = U.golden_2d()
    a = mesh.arrays()
    assert mesh.num_cells == 1024 and mesh.num_vertices == 1089 and mesh.num_faces == 2112
    assert np.abs(a["cell_centroid"].T - z["cell_centroid"]).max() < 1e-15
    np.testing.assert_allclose(a["cell_volume"], 1.0 / 1024, rtol=1e-14)


def test_golden_3d_shock_box(fvh, oracle_lib):
    mesh, z = U.golden_3d()
    a = mesh.arrays()
    assert np.abs(a["cell_centroid"].T - z["std_cell_centroid"]).max() < 1e-13
    p = fvh.make_params(3, cfl=1.0 / 3.0)  # 3d/inputs.cc:101-116
    state = fvh.initial_state("shock_box", mesh, p)
    st, t, n = U.oracle_run(oracle_lib, mesh, state, p, int(z["iterations"]))
    assert st == 0 and n == 12
    assert abs(t - float(z["soln_time"])) <= 1e-14
    cols = U.dump_columns(state, 3)
    expected = np.zeros_like(cols)
    expected[:, 0], expected[:, 1], expected[:, 2] = z["density"], z["internal_energy"], z["pressure"]
    assert U.numdiff_ok(expected, cols, 1e-14)
    assert float(z["max_abs_velocity"]) < 1e-15


def test_ideal_gas_known_answers(fvh, oracle_lib):
    """ideal_gas.cc:40-79: default ideal_gas_t (gamma 2, cv 1, ideal_gas.h:42-44);
    (d, p) = (1, 1), (2, 2) give e = 1, a = sqrt(2), T = 1."""
    d = np.array([1.0, 2.0])
    p = np.array([1.0, 2.0])
    e, T, a = np.zeros(2), np.zeros(2), np.zeros(2)
    dp = C.POINTER(C.c_double)
    oracle_lib.oracle_state_from_pressure(2, 2.0, 1.0, *(x.ctypes.data_as(dp) for x in (d, p, e, T, a)))
    tol = 1e-14  # config::test_tolerance (flecsale-config.h.in)
    assert np.all(np.abs(e - 1.0) <= tol) and np.all(np.abs(T - 1.0) <= tol)
    assert np.all(np.abs(a - np.sqrt(2.0)) <= tol)
    assert np.all(np.abs((2.0 - 1.0) * d * e - p) <= tol)


def test_product_closure_matches_oracle(fvh, oracle_lib):
    """The library's initial-state closure equals the oracle's bit for bit."""
    mesh = fvh.HostMesh.box(2, [7, 5], [0, 0], [1, 1], 0.2, 3)
    prm = fvh.make_params(2, gamma=1.67, cv=0.7)
    s = fvh.initial_state("four_quadrant", mesh, prm)
    nc = mesh.num_cells
    e, T, a = np.zeros(nc), np.zeros(nc), np.zeros(nc)
    dp = C.POINTER(C.c_double)
    d, pr = np.ascontiguousarray(s[0]), np.ascontiguousarray(s[4])
    oracle_lib.oracle_state_from_pressure(nc, 1.67, 0.7, *(x.ctypes.data_as(dp) for x in (d, pr, e, T, a)))
    assert np.array_equal(e, s[3]) and np.array_equal(T, s[5]) and np.array_equal(a, s[6])


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_threads_do_not_change_the_bits(fvh, oracle_lib, dim):
    """The CPU baseline times the oracle on one thread and on all host
    threads; both compute the same bits (cells are independent within a task
    and the dt reduction is a minimum), so the two timings measure the same
    work."""
    if dim == 2:
        mesh = fvh.HostMesh.box(2, (60, 50), [0, 0], [1, 1], 0.2, 3)
        p = fvh.make_params(2, flux="hllc", cfl=0.4, boundary="outflow")
        kind = "four_quadrant"
    else:
        mesh = fvh.HostMesh.box(3, (12, 10, 9), [0, 0, 0], [1, 1, 1], 0.15, 4)
        p = fvh.make_params(3, flux="rusanov", cfl=0.3)
        kind = "inner_cube"
    out = []
    try:
        for threads in (1, 0):
            oracle_lib.oracle_set_threads(threads)
            s = fvh.initial_state(kind, mesh, p)
            st, t, _ = U.oracle_run(oracle_lib, mesh, s, p, 8)
            assert st == 0
            out.append((s, t))
    finally:
        oracle_lib.oracle_set_threads(0)
    assert out[0][1] == out[1][1] and np.array_equal(out[0][0], out[1][0])
