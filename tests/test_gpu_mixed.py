"""Mixed-precision form (FP32 reconstruction/flux, FP64 state/update/dt) against
the FP64 path on the same mesh and initial state.

Tolerance written out: relative L1 density error <= 1e-4 against FP64 (the
stated accuracy bar of the mixed form).  Mass and total energy are conserved to
FP64 roundoff (walls only), because each face flux is accumulated in FP64 with
the same bits on both sides.
"""
import numpy as np
import pytest

import flecsale_gb300.hydro as H

pytestmark = pytest.mark.gpu


def _run(mesh, params, state, nsteps):
    dmesh, dstate = H.DeviceMesh(mesh), H.DeviceState(mesh.dim, mesh.num_cells)
    solver = H.Solver(dmesh, params)
    dstate.upload(state)
    solver.reset(0.0)
    solver.run(dstate, nsteps)
    code, t, cell = solver.status()
    assert code == 0, (code, cell)
    return dstate.download(), t


def _l1(a, b):
    return np.abs(a - b).sum() / np.abs(b).sum()


def _totals(state, vol, dim):
    ke = sum(state[1 + i] ** 2 for i in range(dim))
    return (np.sum(state[0] * vol), np.sum(state[0] * (state[1 + dim] + 0.5 * ke) * vol))


CASES = [
    (2, (128, 96), "four_quadrant", "hllc", "barth_jespersen", 2, 60, "outflow"),
    (2, (128, 96), "kelvin_helmholtz", "hllc", "barth_jespersen", 2, 60),
    (2, (128, 96), "sod", "hlle", "barth_jespersen", 2, 60),
    (2, (100, 10), "sod", "hllc", "barth_jespersen", 1, 60),
    (3, (24, 20, 16), "inner_cube", "rusanov", "barth_jespersen", 2, 20),
    (3, (24, 20, 16), "inner_cube", "hllc", "barth_jespersen", 2, 20, "outflow"),
    # unlimited gradients (the limiter-free kernels)
    (2, (128, 96), "kelvin_helmholtz", "hlle", "none", 2, 20),
    (3, (24, 20, 16), "kelvin_helmholtz", "hllc", "none", 2, 10),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}d-{c[2]}-{c[3]}-{c[4]}-o{c[5]}")
def test_mixed_close_to_fp64(cuda, case):
    dim, n, prob, flux, lim, order, nsteps = case[:7]
    bc = case[7] if len(case) > 7 else "wall"
    mesh = H.HostMesh.box(dim, n, [0] * dim, [1] * dim, 0.2 if dim == 2 else 0.15, 3)
    kw = dict(flux=flux, limiter=lim, order=order, cfl=0.4 if dim == 2 else 0.3, final_time=10.0,
              boundary=bc)
    s0 = H.initial_state(prob, mesh, H.make_params(dim, **kw), seed=5)
    ref, t64 = _run(mesh, H.make_params(dim, **kw), s0, nsteps)
    mix, t32 = _run(mesh, H.make_params(dim, precision="mixed", **kw), s0, nsteps)
    assert abs(t32 - t64) / t64 < 1e-4
    assert _l1(mix[0], ref[0]) <= 1e-4
    E = lambda s: s[0] * (s[1 + dim] + 0.5 * sum(s[1 + i] ** 2 for i in range(dim)))
    assert _l1(E(mix), E(ref)) <= 1e-4
    vol = mesh.arrays()["cell_volume"]
    if bc == "wall":  # closed box: mass and energy conserved to FP64 roundoff
        m0, e0 = _totals(s0, vol, dim)
        m1, e1 = _totals(mix, vol, dim)
        assert abs(m1 - m0) / m0 < 1e-12 and abs(e1 - e0) / e0 < 1e-12


def test_mixed_benchmark_workload_200_steps(cuda):
    """The benchmark workload: 1024^2 jittered four-quadrant, HLLC, CFL 0.4,
    outflow boundaries, 200 steps; mixed vs FP64 relative L1 density <= 1e-4."""
    mesh = H.HostMesh.box(2, (1024, 1024), [0, 0], [1, 1], 0.2, 1)
    kw = dict(flux="hllc", cfl=0.4, final_time=10.0, boundary="outflow")
    s0 = H.initial_state("four_quadrant", mesh, H.make_params(2, **kw))
    ref, _ = _run(mesh, H.make_params(2, **kw), s0, 200)
    mix, _ = _run(mesh, H.make_params(2, precision="mixed", **kw), s0, 200)
    assert _l1(mix[0], ref[0]) <= 1e-4


def test_mixed_deterministic(cuda):
    mesh = H.HostMesh.box(2, (200, 150), [0, 0], [1, 1], 0.2, 8)
    p = H.make_params(2, flux="hllc", cfl=0.4, precision="mixed")
    s0 = H.initial_state("kelvin_helmholtz", mesh, p, seed=2)
    a, _ = _run(mesh, p, s0, 25)
    b, _ = _run(mesh, p, s0, 25)
    assert np.array_equal(a, b)


SHAPES = [(128, 1, 0), (256, 1, 0), (128, 2, 0), (256, 2, 0), (128, 1, 1), (256, 1, 1),
          (128, 2, 1), (128, 3, 0), (256, 4, 1)]
STAGED = 4  # FVH_SCHEDULE_STAGED: gradients from records staged in shared memory (2D)


@pytest.mark.parametrize("dim", [2, 3])
def test_solver_shapes_bitwise_equal(cuda, dim):
    """Every launch shape of the mixed solver gives the same bits, the staged
    gradients (2D) included; autotuning leaves the state, solution time and
    status word as they were."""
    n = (160, 120) if dim == 2 else (20, 18, 16)
    mesh = H.HostMesh.box(dim, n, [0] * dim, [1] * dim, 0.2, 4)
    p = H.make_params(dim, flux="hllc", cfl=0.4 if dim == 2 else 0.3, precision="mixed",
                      boundary="outflow")
    s0 = H.initial_state("four_quadrant" if dim == 2 else "inner_cube", mesh, p, seed=3)
    dmesh = H.DeviceMesh(mesh)
    outs = []
    shapes = SHAPES + ([(128, 1, STAGED), (256, 2, STAGED | 1), (128, 3, STAGED)] if dim == 2 else [])
    if dim == 3:  # no staged gradients in 3D
        with pytest.raises(H.FvhError):
            H.Solver(dmesh, p).set_shape(128, 1, STAGED)
    for shape in shapes:
        dstate = H.DeviceState(dim, mesh.num_cells)
        solver = H.Solver(dmesh, p)
        solver.set_shape(*shape)
        dstate.upload(s0)
        solver.reset(0.0)
        solver.run(dstate, 12)
        code, t, _ = solver.status()
        assert code == 0
        outs.append((dstate.download(), t))
    for s, t in outs[1:]:
        assert t == outs[0][1]
        assert np.array_equal(s, outs[0][0])
    # autotune then run: same bits as the untuned run
    dstate = H.DeviceState(dim, mesh.num_cells)
    solver = H.Solver(dmesh, p)
    dstate.upload(s0)
    solver.reset(0.0)
    best = solver.autotune(dstate, trial_steps=2)
    assert (best["block"], best["cells_per_thread"], best["schedule"] & ~STAGED) in SHAPES
    assert best["ms_per_step"] > 0
    assert np.array_equal(dstate.download(), s0)
    code, t, _ = solver.status()
    assert code == 0 and t == 0.0
    solver.run(dstate, 12)
    assert np.array_equal(dstate.download(), outs[0][0])
    with pytest.raises(H.FvhError):
        solver.set_shape(64, 1, 0)


def _split_cases():
    rng = np.random.default_rng(11)
    f = (rng.uniform(1, 2, 4000) * 2.0 ** rng.integers(-70, 120, 4000)).astype(np.float32)
    f = f * np.where(rng.random(4000) < 0.5, -1, 1).astype(np.float32)
    ulp = np.spacing(np.abs(f)).astype(np.float64)
    fd = f.astype(np.float64)
    ties = fd + 0.5 * ulp                       # exact halfway cases: round to even
    near = fd + 0.5 * ulp * (1 - 2.0 ** -20)    # just below halfway
    carry = 2.0 ** rng.integers(-70, 120, 500) * (1 - 2.0 ** -25)  # rounds up a binade
    rand = rng.standard_normal(20000) * 10.0 ** rng.uniform(-20, 30, 20000)
    special = np.array([0.0, -0.0, 1e-300, -1e-300, 2.0 ** -127, 2.0 ** -100, 1e39, -1e39,
                        np.inf, -np.inf, 1.0, -1.0, 0.1, 1.0 / 3.0])
    return np.concatenate([ties, near, carry, rand, special, fd])


def test_integer_pipe_conversions_exact(cuda):
    """The mixed form's FP64 -> FP32 rounding and FP64 -> double-float split
    run on the integer pipe; they must equal IEEE round-to-nearest-even
    exactly: hi = RN32(x), lo = RN32(x - hi) for |x| >= 2^-74 (lo = 0 below),
    FP32 subnormals flush to zero, hi converts back to FP64 exactly."""
    torch = cuda
    x = _split_cases()
    n = x.size
    xd = torch.from_numpy(x).cuda()
    hi, lo, rn = (torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(3))
    back = torch.empty(n, dtype=torch.float64, device="cuda")
    H.check(H.lib().fvh_debug_split(xd.data_ptr(), n, hi.data_ptr(), lo.data_ptr(),
                                    rn.data_ptr(), back.data_ptr(), None), "fvh_debug_split")
    torch.cuda.synchronize()
    hi, lo, rn, back = (t.cpu().numpy() for t in (hi, lo, rn, back))
    with np.errstate(over="ignore", invalid="ignore"):
        ref = x.astype(np.float32)
        ref_lo = (x - ref.astype(np.float64)).astype(np.float32)
    ax = np.abs(x)
    ref = np.where(ax < 2.0 ** -126, np.copysign(np.float32(0), x), ref).astype(np.float32)
    ref_lo = np.where((ax < 2.0 ** -74) | ~np.isfinite(ref), np.float32(0), ref_lo)
    assert np.array_equal(rn.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(hi.view(np.uint32), ref.view(np.uint32))
    fin = np.isfinite(ref)
    assert np.array_equal(np.abs(lo[fin]), np.abs(ref_lo[fin]))
    assert np.array_equal(lo[fin] == 0, ref_lo[fin] == 0)
    assert np.array_equal(np.sign(lo[fin]), np.sign(ref_lo[fin]))
    assert np.array_equal(back[fin], ref[fin].astype(np.float64))
    nan = np.array([np.nan])
    xd = torch.from_numpy(nan).cuda()
    h1, l1, r1 = (torch.empty(1, dtype=torch.float32, device="cuda") for _ in range(3))
    b1 = torch.empty(1, dtype=torch.float64, device="cuda")
    H.check(H.lib().fvh_debug_split(xd.data_ptr(), 1, h1.data_ptr(), l1.data_ptr(),
                                    r1.data_ptr(), b1.data_ptr(), None), "fvh_debug_split")
    assert np.isnan(r1.cpu().numpy()[0]) and np.isnan(h1.cpu().numpy()[0])


@pytest.mark.parametrize("dim,schedule,final_time", [(2, 0, 10.0), (2, 1, 10.0), (3, 1, 10.0),
                                                     (2, 1, 0.02)])
def test_run_equals_single_steps_bitwise(cuda, dim, schedule, final_time):
    """Inside fvh_solver_run each corrector prepares the next step's FP32 pack
    and dt; the result must be bitwise that of the same number of single
    steps (each recomputing pack and dt from the FP64 state), also when the
    run passes the final time (dt = 0 steps leave the state untouched)."""
    torch = cuda
    n = (96, 80) if dim == 2 else (16, 14, 12)
    mesh = H.HostMesh.box(dim, n, [0] * dim, [1] * dim, 0.2, 6)
    p = H.make_params(dim, flux="hllc", cfl=0.4 if dim == 2 else 0.3, precision="mixed",
                      boundary="outflow", final_time=final_time)
    s0 = H.initial_state("four_quadrant" if dim == 2 else "inner_cube", mesh, p, seed=4)
    dmesh = H.DeviceMesh(mesh)
    stream = torch.cuda.Stream()
    out = []
    for mode in ("run", "steps", "run_default_stream"):
        ds = H.DeviceState(dim, mesh.num_cells)
        sol = H.Solver(dmesh, p)
        sol.set_shape(128, 1, schedule)
        st = None if mode == "run_default_stream" else stream
        ds.upload(s0, st)
        sol.reset(0.0, st)
        if mode == "steps":
            for _ in range(25):
                sol.step(ds, st)
        else:
            sol.run(ds, 25, stream=st)
        code, t, _ = sol.status(st)
        assert code == 0
        out.append((ds.download(st), t))
    for s, t in out[1:]:
        assert t == out[0][1]
        assert np.array_equal(s, out[0][0])
    if final_time < 1:
        assert out[0][1] == final_time


@pytest.mark.parametrize("dim,n,schedule,nsteps,precision", [
    (2, (120, 100), 0, 1, "mixed"), (2, (120, 100), 0, 4, "mixed"),
    (2, (320, 256), 1, 1, "mixed"), (2, (320, 256), 1, 3, "mixed"),
    (3, (44, 40, 38), 1, 2, "mixed"),
    (2, (120, 100), 0, 1, "fp64"), (2, (320, 256), 0, 3, "fp64"),
    (3, (44, 40, 38), 0, 2, "fp64")])
def test_advance_host_pinned_equals_copies(cuda, dim, n, schedule, nsteps, precision):
    """fvh_solver_advance_host with pinned host planes (kernels read and write
    host memory directly) gives the same bits as with pageable planes (copies)
    and as upload + run + download; the device state ends up the same too.
    The FP64 form does not copy up the temperature plane: a garbage
    temperature in the pinned planes must not change anything."""
    torch = cuda
    mesh = H.HostMesh.box(dim, n, [0] * dim, [1] * dim, 0.2 if dim == 2 else 0.15, 9)
    prob = "four_quadrant" if dim == 2 else "inner_cube"
    p = H.make_params(dim, flux="hllc", cfl=0.4 if dim == 2 else 0.3, precision=precision,
                      boundary="outflow")
    s0 = H.initial_state(prob, mesh, p, seed=1)
    dmesh = H.DeviceMesh(mesh)
    stream = torch.cuda.Stream()
    nc = mesh.num_cells
    np_ = 5 + dim
    res = []
    for kind in ("pinned", "pageable", "run"):
        ds = H.DeviceState(dim, nc)
        sol = H.Solver(dmesh, p)
        if precision == "mixed":
            sol.set_shape(128, 1, schedule)
        if kind == "run":
            ds.upload(s0, stream)
            sol.reset(0.125, stream)
            sol.run(ds, nsteps, stream=stream)
            host, t = ds.download(stream), sol.soln_time(stream)
        else:
            if kind == "pinned":
                host = torch.empty((np_, nc), dtype=torch.float64, pin_memory=True).numpy()
            else:
                host = np.empty((np_, nc), np.float64)
            host[:] = s0[:np_]
            if kind == "pinned" and precision == "fp64":
                host[dim + 3] = np.nan
            t = sol.advance_host(ds, host, nsteps, 0.125, stream)
        res.append((host.copy(), t, ds.download(stream)))
    for h, t, d in res[1:]:
        assert t == res[0][1]
        assert np.array_equal(h, res[0][0])
        assert np.array_equal(d, res[0][2])
    assert not np.array_equal(res[0][0], s0[:np_])


@pytest.mark.parametrize("dim", [2, 3])
def test_colour_schedule(cuda, dim):
    """Schedule 2 (face colouring): deterministic, conservative, within
    1e-10 relative L1 of the gather schedules (its sums add each cell's
    fluxes in colour order), and a run equals single steps bitwise."""
    torch = cuda
    n = (90, 70) if dim == 2 else (14, 12, 10)
    mesh = H.HostMesh.box(dim, n, [0] * dim, [1] * dim, 0.2 if dim == 2 else 0.15, 8)
    for bc in ("outflow", "wall"):
        p = H.make_params(dim, flux="hllc", cfl=0.4 if dim == 2 else 0.3, precision="mixed",
                          boundary=bc)
        s0 = H.initial_state("four_quadrant" if dim == 2 else "inner_cube", mesh, p, seed=5)
        dmesh = H.DeviceMesh(mesh)
        stream = torch.cuda.Stream()
        out = {}
        for label, shape, mode in (("gather", (128, 1, 1), "run"), ("colour", (128, 1, 2), "run"),
                                   ("colour2", (256, 1, 2), "run"),
                                   ("colour_steps", (128, 1, 2), "steps")):
            ds = H.DeviceState(dim, mesh.num_cells)
            sol = H.Solver(dmesh, p)
            sol.set_shape(*shape)
            ds.upload(s0, stream)
            sol.reset(0.0, stream)
            if mode == "run":
                sol.run(ds, 16, stream=stream)
            else:
                for _ in range(16):
                    sol.step(ds, stream)
            code, t, _ = sol.status(stream)
            assert code == 0
            out[label] = (ds.download(stream), t)
        g, c = out["gather"][0], out["colour"][0]
        assert np.abs(c[0] - g[0]).sum() / np.abs(g[0]).sum() <= 1e-10
        assert np.array_equal(out["colour"][0], out["colour2"][0])
        assert np.array_equal(out["colour"][0], out["colour_steps"][0])
        if bc == "wall":
            vol = mesh.arrays()["cell_volume"]
            m0, e0 = _totals(s0, vol, dim)
            m1, e1 = _totals(c, vol, dim)
            assert abs(m1 - m0) / m0 < 1e-12 and abs(e1 - e0) / e0 < 1e-12
