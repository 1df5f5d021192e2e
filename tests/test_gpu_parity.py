"""GPU parity of the plain FP64 path against the oracle, through the C ABI.

The FP64 kernels follow the reference's arithmetic order and are compiled
without contraction, so every comparison here is bitwise (np.array_equal), which
is stricter than the 1e-11 relative bar; the few places that also check 1e-11
say so.
"""
import ctypes as C

import numpy as np
import pytest

import flecsale_gb300.hydro as H
from tests import _util as U

pytestmark = pytest.mark.gpu

CASES = [
    # dim, n, jitter, problem, flux, limiter, order, swap[, boundary]
    (2, (24, 17), 0.2, "four_quadrant", "hllc", "barth_jespersen", 2, True, "outflow"),
    (2, (24, 17), 0.2, "four_quadrant", "rusanov", "barth_jespersen", 2, True, "outflow"),
    (3, (7, 6, 5), 0.15, "inner_cube", "hllc", "barth_jespersen", 2, True, "outflow"),
    (2, (24, 17), 0.2, "four_quadrant", "hllc", "barth_jespersen", 2, True),
    (2, (24, 17), 0.2, "four_quadrant", "hlle", "barth_jespersen", 2, True),
    (2, (24, 17), 0.2, "kelvin_helmholtz", "rusanov", "barth_jespersen", 2, False),
    (2, (24, 17), 0.2, "four_quadrant", "hllc", "none", 2, True),
    (2, (24, 17), 0.2, "kelvin_helmholtz", "hlle", "none", 2, False),
    (2, (24, 17), 0.2, "sod", "hllc", "barth_jespersen", 2, True),
    (2, (24, 17), 0.0, "sod", "hllc", "barth_jespersen", 1, True),
    (3, (7, 6, 5), 0.15, "inner_cube", "rusanov", "barth_jespersen", 2, True),
    (3, (7, 6, 5), 0.15, "inner_cube", "hlle", "barth_jespersen", 2, True),
    (3, (7, 6, 5), 0.15, "kelvin_helmholtz", "hllc", "none", 2, False),
    (3, (7, 6, 5), 0.15, "inner_cube", "hllc", "barth_jespersen", 1, True),
]


def _setup(cuda, dim, n, jitter, problem, flux, limiter, order, swap, boundary="wall",
           warm_steps=2):
    mesh = H.HostMesh.box(dim, n, [0] * dim, [1] * dim, jitter, 7)
    p = H.make_params(dim, flux=flux, limiter=limiter, order=order, swap=swap, cfl=0.4,
                      boundary=boundary)
    state = H.initial_state(problem, mesh, p, seed=11)
    O = __import__("oracle").load()
    # advance a little on the oracle so gradients and limiters are active
    st, _, _ = U.oracle_run(O, mesh, state, p, warm_steps)
    assert st == 0 and np.all(np.isfinite(state[:5 + dim]))
    return mesh, p, state, O


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}d-{c[3]}-{c[4]}-{c[5]}-o{c[6]}-s{int(c[7])}"
                         + (f"-{c[8]}" if len(c) > 8 else ""))
def test_tasks_bitwise(cuda, case):
    torch = cuda
    dim = case[0]
    mesh, p, state, O = _setup(cuda, *case)
    dmesh = H.DeviceMesh(mesh)
    stream = torch.cuda.Stream()
    sh = H.stream_handle(stream)
    nc, nf = mesh.num_cells, mesh.num_faces
    ds = torch.tensor(state, device="cuda")
    dg = torch.zeros((U.grad_rows(dim), nc), dtype=torch.float64, device="cuda")
    df = torch.zeros((dim + 2, nf), dtype=torch.float64, device="cuda")
    scal = torch.tensor([0.05, 0.0], dtype=torch.float64, device="cuda")  # soln time, dt
    ws_bytes = H.lib().fvh_time_step_workspace_bytes(nc)
    ws = torch.zeros(ws_bytes // 8 + 1, dtype=torch.float64, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    sv, gv, fv = U.device_state_view(ds, dim), U.device_gradient_view(dg, dim), U.device_flux_view(df, dim)
    torch.cuda.synchronize()
    L = H.lib()
    # time step
    H.check(L.fvh_evaluate_time_step(C.byref(dmesh.view), C.byref(sv), C.byref(p), scal.data_ptr(),
                                     scal.data_ptr() + 8, ws.data_ptr(), ws_bytes, status.data_ptr(), sh))
    # gradients, fluxes, update
    H.check(L.fvh_evaluate_gradients(C.byref(dmesh.view), C.byref(sv), C.byref(gv), C.byref(p), sh))
    H.check(L.fvh_evaluate_fluxes(C.byref(dmesh.view), C.byref(sv), C.byref(gv), C.byref(fv), C.byref(p), sh))
    g_gpu, f_gpu = None, None
    stream.synchronize()
    g_gpu, f_gpu = dg.cpu().numpy(), df.cpu().numpy()
    H.check(L.fvh_apply_update(C.byref(dmesh.view), C.byref(p), scal.data_ptr() + 8, 0.5, C.byref(fv),
                               C.byref(sv), scal.data_ptr(), status.data_ptr(), sh))
    stream.synchronize()
    t_gpu, dt_gpu = scal.cpu().numpy()
    s_gpu = ds.cpu().numpy()
    assert int(status.item()) == -1  # FVH_STATUS_CLEAR

    st, dt = U.oracle_time_step(O, mesh, state, p, 0.05)
    assert st == 0 and dt_gpu == dt
    g = U.oracle_gradients(O, mesh, state, p)
    assert np.array_equal(g_gpu, g, equal_nan=True)
    f = U.oracle_fluxes(O, mesh, state, g, p)
    assert np.array_equal(f_gpu, f, equal_nan=True)
    st, t, _ = U.oracle_update(O, mesh, state, f, p, dt, 0.5, 0.05)
    assert st == 0 and t_gpu == t
    assert np.array_equal(s_gpu[:5 + dim], state[:5 + dim], equal_nan=True)


@pytest.mark.parametrize("dim", [2, 3])
def test_solver_run_bitwise(cuda, dim):
    if dim == 2:
        mesh = H.HostMesh.box(2, (64, 48), [0, 0], [1, 1], 0.2, 1)
        p = H.make_params(2, flux="hllc", cfl=0.4, boundary="outflow")
        state = H.initial_state("four_quadrant", mesh, p)
        nsteps = 30
    else:
        mesh = H.HostMesh.box(3, (12, 11, 10), [0, 0, 0], [1, 1, 1], 0.15, 2)
        p = H.make_params(3, flux="rusanov", cfl=0.3)
        state = H.initial_state("inner_cube", mesh, p)
        nsteps = 10
    O = __import__("oracle").load()
    dmesh, dstate = H.DeviceMesh(mesh), H.DeviceState(dim, mesh.num_cells)
    solver = H.Solver(dmesh, p)
    torch = cuda
    stream = torch.cuda.Stream()
    dstate.upload(state, stream)
    solver.reset(0.0, stream)
    assert solver.run(dstate, nsteps, stream=stream) == nsteps
    out = dstate.download(stream)
    stream.synchronize()
    code, t_gpu, _ = solver.status(stream)
    assert code == 0
    st, t, n = U.oracle_run(O, mesh, state, p, nsteps)
    assert st == 0 and n == nsteps and t_gpu == t
    assert np.array_equal(out, state)
    # the stated bar, written out: <= 1e-11 relative per cell
    rel = np.abs(out - state) / np.maximum(np.abs(state), 1e-300)
    assert rel.max() <= 1e-11


def test_gpu_golden_2d(cuda):
    mesh, z = U.golden_2d()
    p = H.make_params(2)
    state = H.initial_state("shock_box", mesh, p)
    dmesh, dstate = H.DeviceMesh(mesh), H.DeviceState(2, mesh.num_cells)
    solver = H.Solver(dmesh, p)
    dstate.upload(state)
    solver.reset(0.0)
    solver.run(dstate, int(z["iterations"]))
    out = dstate.download()
    code, t, _ = solver.status()
    assert code == 0 and abs(t - float(z["soln_time"])) <= 1e-14
    assert U.numdiff_ok(z["cells"], U.dump_columns(out, 2), 1e-14)
    # the reference's two-rank run of the same problem, cell by cell
    assert U.two_rank_max_diff(U.dump_columns(out, 2), z["cell_centroid"], U.two_rank_dumps()) <= 1e-14
    O = __import__("oracle").load()
    U.oracle_run(O, mesh, state, p, 20)
    assert np.array_equal(out, state)


def test_gpu_golden_3d(cuda):
    mesh, z = U.golden_3d()
    p = H.make_params(3, cfl=1.0 / 3.0)
    state = H.initial_state("shock_box", mesh, p)
    dmesh, dstate = H.DeviceMesh(mesh), H.DeviceState(3, mesh.num_cells)
    solver = H.Solver(dmesh, p)
    dstate.upload(state)
    solver.reset(0.0)
    solver.run(dstate, int(z["iterations"]))
    out = dstate.download()
    code, t, _ = solver.status()
    assert code == 0 and abs(t - float(z["soln_time"])) <= 1e-14
    cols = U.dump_columns(out, 3)
    exp = np.zeros_like(cols)
    exp[:, 0], exp[:, 1], exp[:, 2] = z["density"], z["internal_energy"], z["pressure"]
    assert U.numdiff_ok(exp, cols, 1e-14)


def test_stop_at_final_time(cuda):
    """Sod 100x10 first-order HLLC to t = 0.2 (stop when t >= t_f)."""
    mesh = H.HostMesh.box(2, (100, 10), [0, 0], [1, 0.1], 0.0, 0)
    p = H.make_params(2, flux="hllc", order=1, cfl=0.5, final_time=0.2)
    state = H.initial_state("sod", mesh, p)
    dmesh, dstate = H.DeviceMesh(mesh), H.DeviceState(2, mesh.num_cells)
    solver = H.Solver(dmesh, p)
    dstate.upload(state)
    solver.reset(0.0)
    n = solver.run(dstate, 10000, stop_at_final_time=True, check_every=1)
    out = dstate.download()
    code, t, _ = solver.status()
    O = __import__("oracle").load()
    st, t_o, n_o = U.oracle_run(O, mesh, state, p, 10000, stop_at_final=True)
    assert code == 0 and st == 0 and n == n_o and t == t_o
    assert abs(t - 0.2) < 1e-12
    assert np.array_equal(out, state)


def test_negative_state_is_reported(cuda):
    """A host-injected negative internal energy is reported with its cell id,
    the reference's THROW at tasks.h:654-655, without touching other cells."""
    mesh = H.HostMesh.box(2, (16, 16), [0, 0], [1, 1], 0.1, 3)
    p = H.make_params(2)
    state = H.initial_state("uniform", mesh, p)
    bad = [77, 200]
    for c in bad:
        state[3, c] = -1.0  # internal energy
    torch = cuda
    dim, nc, nf = 2, mesh.num_cells, mesh.num_faces
    dmesh = H.DeviceMesh(mesh)
    ds = torch.tensor(state, device="cuda")
    df = torch.zeros((dim + 2, nf), dtype=torch.float64, device="cuda")
    scal = torch.tensor([0.0, 1e-3], dtype=torch.float64, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    H.check(H.lib().fvh_apply_update(C.byref(dmesh.view), C.byref(p), scal.data_ptr() + 8, 0.5,
                                     C.byref(U.device_flux_view(df, dim)), C.byref(U.device_state_view(ds, dim)),
                                     scal.data_ptr(), status.data_ptr(), None))
    torch.cuda.synchronize()
    code, cell = C.c_int32(), C.c_int64()
    H.lib().fvh_status_decode(int(status.item()) & ((1 << 64) - 1), C.byref(code), C.byref(cell))
    assert code.value == H.ERR_NEGATIVE_STATE and cell.value == min(bad)
    O = __import__("oracle").load()
    st, _, bad_o = U.oracle_update(O, mesh, state, np.zeros((dim + 2, nf)), p, 1e-3, 0.5)
    assert st == H.ERR_NEGATIVE_STATE and bad_o == min(bad)
    out = ds.cpu().numpy()
    ok = np.ones(nc, bool)
    ok[bad] = False
    assert np.array_equal(out[:, ok], state[:, ok])


def test_infinite_dt_is_reported(cuda):
    """Zero sound speed and velocity: the reference throws "infinite delta t"
    (tasks.h:366-367); the device status records it."""
    mesh = H.HostMesh.box(2, (8, 8), [0, 0], [1, 1], 0.0, 0)
    p = H.make_params(2)
    torch = cuda
    state = np.zeros((8, mesh.num_cells))
    state[0] = 1.0
    ds = torch.tensor(state, device="cuda")
    dmesh = H.DeviceMesh(mesh)
    scal = torch.zeros(2, dtype=torch.float64, device="cuda")
    nb = H.lib().fvh_time_step_workspace_bytes(mesh.num_cells)
    ws = torch.zeros(nb // 8 + 1, dtype=torch.float64, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    H.check(H.lib().fvh_evaluate_time_step(C.byref(dmesh.view), C.byref(U.device_state_view(ds, 2)),
                                           C.byref(p), scal.data_ptr(), scal.data_ptr() + 8, ws.data_ptr(),
                                           nb, status.data_ptr(), None))
    torch.cuda.synchronize()
    code = C.c_int32()
    H.lib().fvh_status_decode(int(status.item()) & ((1 << 64) - 1), C.byref(code), None)
    assert code.value == H.ERR_INFINITE_DT


def test_full_size_four_quadrant_bitwise_and_conservative(cuda):
    """1024^2 jittered four-quadrant (the benchmark workload), 2 steps: bitwise
    equal to the oracle; mass and energy conserved (walls only) to roundoff."""
    mesh = H.HostMesh.box(2, (1024, 1024), [0, 0], [1, 1], 0.2, 1)
    p = H.make_params(2, flux="hllc", cfl=0.4)  # walls: mass and energy stay in the box
    state = H.initial_state("four_quadrant", mesh, p)
    vol = mesh.arrays()["cell_volume"]
    m0 = np.sum(state[0] * vol)
    E0 = np.sum(state[0] * (state[3] + 0.5 * (state[1] ** 2 + state[2] ** 2)) * vol)
    dmesh, dstate = H.DeviceMesh(mesh), H.DeviceState(2, mesh.num_cells)
    solver = H.Solver(dmesh, p)
    dstate.upload(state)
    solver.reset(0.0)
    solver.run(dstate, 2)
    out = dstate.download()
    assert solver.status()[0] == 0
    m1 = np.sum(out[0] * vol)
    E1 = np.sum(out[0] * (out[3] + 0.5 * (out[1] ** 2 + out[2] ** 2)) * vol)
    assert abs(m1 - m0) / m0 < 1e-13 and abs(E1 - E0) / E0 < 1e-13
    O = __import__("oracle").load()
    U.oracle_run(O, mesh, state, p, 2)
    assert np.array_equal(out, state)


def _gpu_run(mesh, p, state, nsteps):
    dmesh, dstate = H.DeviceMesh(mesh), H.DeviceState(mesh.dim, mesh.num_cells)
    solver = H.Solver(dmesh, p)
    dstate.upload(state)
    solver.reset(0.0)
    assert solver.run(dstate, nsteps) == nsteps
    code, t, cell = solver.status()
    assert code == 0, (code, cell)
    return dstate.download(), t


def _l1(a, b):
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def _energy(s, dim):
    return s[0] * (s[1 + dim] + 0.5 * sum(s[1 + i] ** 2 for i in range(dim)))


def test_benchmark_workload_200_steps_against_oracle(cuda):
    """The benchmark workload at its own length: 1024^2 jittered (+-0.2h, seed
    1) four-quadrant, HLLC, Barth-Jespersen, CFL 0.4, transmissive boundaries,
    200 steps.  FP64 is bitwise equal to the oracle; the mixed form is within
    relative L1 1e-4 of the oracle in density and total energy."""
    mesh = H.HostMesh.box(2, (1024, 1024), [0, 0], [1, 1], 0.2, 1)
    kw = dict(flux="hllc", cfl=0.4, final_time=1.0e9, boundary="outflow")
    p = H.make_params(2, **kw)
    s0 = H.initial_state("four_quadrant", mesh, p)
    out, t_gpu = _gpu_run(mesh, p, s0, 200)
    mix, t_mix = _gpu_run(mesh, H.make_params(2, precision="mixed", **kw), s0, 200)
    O = __import__("oracle").load()
    ref = s0.copy()
    st, t, n = U.oracle_run(O, mesh, ref, p, 200)
    assert st == 0 and n == 200 and t_gpu == t
    assert np.array_equal(out, ref)
    assert abs(t_mix - t) / t < 1e-4
    assert _l1(mix[0], ref[0]) <= 1e-4 and _l1(_energy(mix, 2), _energy(ref, 2)) <= 1e-4


def test_3d_shock_box_64cube_20_steps_against_oracle(cuda):
    """The 3D shock box of the benchmark at 64^3 (262,144 hexes, jitter
    +-0.15h, seed 2): inner cube, Rusanov, CFL 0.3, walls, 20 steps.  FP64
    bitwise equal to the oracle; mixed within relative L1 1e-4."""
    mesh = H.HostMesh.box(3, (64, 64, 64), [0, 0, 0], [1, 1, 1], 0.15, 2)
    kw = dict(flux="rusanov", cfl=0.3, final_time=1.0e9)
    p = H.make_params(3, **kw)
    s0 = H.initial_state("inner_cube", mesh, p)
    out, t_gpu = _gpu_run(mesh, p, s0, 20)
    mix, _ = _gpu_run(mesh, H.make_params(3, precision="mixed", **kw), s0, 20)
    O = __import__("oracle").load()
    ref = s0.copy()
    st, t, n = U.oracle_run(O, mesh, ref, p, 20)
    assert st == 0 and n == 20 and t_gpu == t
    assert np.array_equal(out, ref)
    assert _l1(mix[0], ref[0]) <= 1e-4 and _l1(_energy(mix, 3), _energy(ref, 3)) <= 1e-4


def test_deterministic_rerun(cuda):
    mesh = H.HostMesh.box(2, (96, 80), [0, 0], [1, 1], 0.2, 5)
    p = H.make_params(2, flux="hllc", cfl=0.4)
    s0 = H.initial_state("kelvin_helmholtz", mesh, p, seed=9)
    outs = []
    for _ in range(2):
        dmesh, dstate = H.DeviceMesh(mesh), H.DeviceState(2, mesh.num_cells)
        solver = H.Solver(dmesh, p)
        dstate.upload(s0)
        solver.reset(0.0)
        solver.run(dstate, 15)
        outs.append(dstate.download())
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("dim,flux,scale", [(2, "hllc", 1e-170), (2, "hllc", 2.0 ** -495),
                                            (2, "hlle", 1e170), (3, "rusanov", 1e-170)])
def test_extreme_magnitudes_take_the_fp64_redo_bitwise(cuda, dim, flux, scale):
    """Density and pressure scaled by `scale` (the Euler equations are
    invariant under rho, p -> s rho, s p: e, T, a and v keep their values).
    With 1e-170 and 1e170 nearly every product has an operand outside the
    2^+-500 range of the integer-pipe arithmetic, so the units of work (dt,
    gradients, face fluxes, updates) are evaluated again with the FP64
    instructions; with 2^-495 only the units whose operands fall below 2^-500
    are.  The runs are bitwise equal to the oracle."""
    if dim == 2:
        mesh = H.HostMesh.box(2, (40, 32), [0, 0], [1, 1], 0.2, 3)
        problem, kw = "four_quadrant", dict(boundary="outflow")
    else:
        mesh = H.HostMesh.box(3, (10, 9, 8), [0, 0, 0], [1, 1, 1], 0.15, 3)
        problem, kw = "inner_cube", {}
    # textbook reconstruction: the reference's e/p gradient swap mixes a
    # scaled and an unscaled variable, which the scaling would turn negative
    p = H.make_params(dim, flux=flux, cfl=0.4, swap=False, **kw)
    state = H.initial_state(problem, mesh, p)
    plain = state.copy()
    for row in (0, dim + 2):  # density, pressure
        state[row] *= scale
    out, t_gpu = _gpu_run(mesh, p, state, 6)
    O = __import__("oracle").load()
    ref = state.copy()
    st, t, n = U.oracle_run(O, mesh, ref, p, 6)
    assert st == 0 and n == 6 and t_gpu == t
    assert np.array_equal(out, ref)
    # a large scale leaves the solution the plain one's, scaled (to rounding);
    # below 1 the limiter's absolute tolerance (1e-9, tasks.h:267-299) lets
    # the tiny density differences go unlimited, so the solutions differ
    if scale > 1:
        st, _, _ = U.oracle_run(O, mesh, plain, p, 6)
        assert st == 0
        assert np.allclose(out[0] / scale, plain[0], rtol=1e-8, atol=0)
