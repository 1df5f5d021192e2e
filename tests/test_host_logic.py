"""Host-side logic that needs no GPU: the serving request stream, the bench's
algorithmic-byte model and its reporting helpers."""
import numpy as np

import flecsale_gb300.hydro as H
from flecsale_gb300 import serve


def test_poisson_requests_deterministic_and_in_range():
    a = serve.poisson_requests(5.0, 30.0, seed=4)
    b = serve.poisson_requests(5.0, 30.0, seed=4)
    assert [(r.arrival, r.side, r.t_end, r.seed) for r in a] == \
           [(r.arrival, r.side, r.t_end, r.seed) for r in b]
    assert 100 < len(a) < 200                       # ~ rate * duration
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0) and arr[-1] < 30.0
    sides = np.array([r.side for r in a])
    assert sides.min() >= 64 and sides.max() <= 2048
    # log-uniform sides: the median side is near the geometric mean
    assert 250 < np.median(sides) < 500
    tend = np.array([r.t_end for r in a])
    assert tend.min() >= 0.05 and tend.max() <= 0.3
    assert {r.kind for r in a} == {"kelvin_helmholtz", "four_quadrant", "sod"}


def test_server_params_scheme():
    p = serve.server_params()
    assert p.precision == H.PRECISION["mixed"] and p.flux_kind == H.FLUX["hllc"]
    assert p.recon_swap_ep == 0 and p.boundary == 1 and p.cfl == 0.4


def test_admission_by_capacity():
    """_fits admits a request while the running set plus it stays within
    every capacity (cells, faces, vertices, problems)."""
    srv = serve.Server.__new__(serve.Server)
    srv.caps = (1000, 2200, 1200, 3)
    reqs = [serve.build_mesh(serve.Request(k, 0.0, s, "sod", 0.1)) for k, s in
            enumerate((20, 20, 10, 5))]
    assert srv._fits([], reqs[0])                       # 400 cells
    assert srv._fits([reqs[0]], reqs[1])                # 800
    assert not srv._fits(reqs[:2], reqs[0])             # 1200 cells > 1000
    assert srv._fits(reqs[:2], reqs[2])                 # 900 cells, 3 problems
    assert not srv._fits(reqs[:3], reqs[3])             # a 4th problem


def test_algorithmic_bytes_model():
    import bench
    m = H.HostMesh.box(2, (64, 48), [0, 0], [1, 1], 0.2, 1)
    b = bench.algorithmic_bytes(m, "mixed")
    assert all(v > 0 for v in b.values())
    # a run's step (no pack_dt) moves less than a single step
    single = b["pack_dt"] + 2 * b["gradients"] + b["flux_update_predictor"] + b["flux_update_corrector"]
    assert bench.per_zone_update_bytes(m, "mixed") * m.num_cells < single
    b64 = bench.algorithmic_bytes(m, "fp64")
    f = bench.per_zone_update_bytes(m, "fp64")
    assert 1300 < f < 1700                              # the 2D figure derived for the reference dataflow
    assert b64["gradients"] > b64["update"]
    m3 = H.HostMesh.box(3, (8, 8, 8), [0, 0, 0], [1, 1, 1], 0.1, 1)
    assert bench.per_zone_update_bytes(m3, "fp64") > f  # 3D moves more per zone-update


def test_roofline_3d_from_a_profile():
    """The 3D roofline: the dominant kernel by time share, its duration scaled
    to the in-run step, the gradients task's reference-dataflow bytes (about
    412 B/cell for hexes with 26 neighbours) over that duration."""
    import bench
    m3 = H.HostMesh.box(3, (8, 8, 8), [0, 0, 0], [1, 1, 1], 0.1, 1)
    prof = {"pack_dt": (0.2, 0.25), "gradients": (1.0, 2.0), "face_flux": (0.5, 2.0),
            "gather_update": (0.4, 2.0)}
    r = bench.roofline_3d(m3, "mixed", prof, in_run_step_ms=(0.05 + 2.0 + 1.0 + 0.8) / 2)
    assert r["kernel"] == "gradients"
    assert abs(r["duration_ms"] - 0.5) < 1e-12      # profiled 1.0 ms, step scaled by 1/2
    sb = bench.algorithmic_bytes(m3, "fp64")["gradients"]
    assert r["algorithmic_bytes_per_launch"] == sb
    assert abs(r["achieved"] - sb / 0.5e-3 / 1e9) < 1e-9
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert abs(sum(k["share"] for k in r["kernels"].values()) - 1.0) < 1e-12


def test_max_over_ranks_without_a_group():
    import bench
    assert bench.max_over_ranks(None, 3.5) == 3.5


def test_reference_arm_json_line():
    """bench.py --impl reference (the CPU reference arm) prints one JSON line
    with the contract's keys, on a small mesh."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--n", "48"], cwd=root, capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 1
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["cells"] == 48 * 48


def test_reference_arm_loads_no_product_code():
    """The reference arm builds its mesh, initial state and parameters with the
    oracle's own code: the process never imports the product package nor maps
    its shared library."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', "
            "'--warmup', '3', '--n', '32']; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "assert 'libflecsale_gb300' not in maps, 'product library mapped'; "
            "assert not [m for m in sys.modules if m.startswith('flecsale_gb300')], "
            "'product package imported'; print('clean')")
    out = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip().endswith("clean")


def test_binding_checks_plane_shapes_before_the_call():
    """The C ABI reads (and advance_host writes) all (5+dim) x num_cells
    doubles of a host state: the binding refuses smaller, larger, strided,
    read-only or mistyped arrays before anything reaches the library."""
    import pytest
    good = np.zeros((7, 10))
    assert H._state_planes(good, 2, 10, "t") is not None
    assert H._state_planes(good, 2, 10, "t", writable=True) is good
    for bad in (np.zeros((7, 9)), np.zeros((6, 10)), np.zeros((8, 10)), np.zeros(70)):
        with pytest.raises(ValueError):
            H._state_planes(bad, 2, 10, "t")
    with pytest.raises(TypeError):
        H._state_planes(np.zeros((7, 20))[:, ::2], 2, 10, "t", writable=True)
    with pytest.raises(TypeError):
        H._state_planes(np.zeros((7, 10), np.float32), 2, 10, "t", writable=True)
    ro = np.zeros((7, 10))
    ro.flags.writeable = False
    with pytest.raises(TypeError):
        H._state_planes(ro, 2, 10, "t", writable=True)
    # read-only use converts a float32 array instead of refusing it
    assert H._state_planes(np.zeros((8, 4), np.float32), 3, 4, "t").dtype == np.float64
    with pytest.raises(TypeError):
        H._dptr(np.zeros(4, np.float32))
    with pytest.raises(TypeError):
        H._iptr(np.zeros(4, np.int64))
    with pytest.raises(TypeError):
        H._dptr(np.zeros((4, 4))[:, 1])


def test_write_dump_refuses_short_planes(tmp_path):
    import pytest
    mesh = H.HostMesh.box(2, (4, 3), [0, 0], [1, 1])
    with pytest.raises(ValueError):
        H.write_dump(str(tmp_path / "d.txt"), mesh, np.zeros((7, mesh.num_cells - 1)), 0.0, 0)
    assert not (tmp_path / "d.txt").exists()


def test_bench_conservation_totals(oracle_lib):
    """The bench's conservation totals: exact for a uniform state, and mass
    and energy kept to rounding by an oracle run between walls."""
    import bench
    from tests import _util as U
    mesh = H.HostMesh.box(2, (20, 16), [0, 0], [2, 1], 0.2, 5)
    p = H.make_params(2, flux="hllc", cfl=0.4)
    n = mesh.num_cells
    s = H.state_from_dvp(2, np.full(n, 2.0), np.stack([np.full(n, 0.5), np.full(n, -1.0)]),
                         np.full(n, 0.8), p.gamma, p.cv)
    tot = bench.conservation_totals(mesh, s)
    e = 0.8 / (2.0 * 0.4)
    assert abs(tot["mass"] - 4.0) <= 1e-13
    assert np.allclose(tot["momentum"], [2.0, -4.0], rtol=1e-13)
    assert abs(tot["energy"] - 4.0 * (e + 0.5 * 1.25)) <= 1e-12
    s = H.initial_state("four_quadrant", mesh, p)
    t0 = bench.conservation_totals(mesh, s)
    st, _, _ = U.oracle_run(oracle_lib, mesh, s, p, 10)
    t1 = bench.conservation_totals(mesh, s)
    assert st == 0
    assert abs(t1["mass"] - t0["mass"]) <= 1e-13 * t0["mass"]
    assert abs(t1["energy"] - t0["energy"]) <= 1e-13 * t0["energy"]


def test_serving_loop_bookkeeping_with_a_fake_batch(monkeypatch):
    """The continuous-batching loop on the host, with the device batch and
    device meshes replaced by fakes that advance each problem's time: every
    request finishes with its own state, running problems are carried into
    each reassignment by the right keep index, and admissions wait for
    capacity."""
    DT = 0.01
    assigns = []

    class FakeDeviceMesh:
        def __init__(self, mesh):
            self.num_cells = mesh.num_cells

    class FakeBatch:
        def __init__(self, params, max_cells, max_faces, max_vertices, max_problems):
            self.problems, self.meshes = [], []

        def query(self, stream=None):
            t = np.array([q["t"] for q in self.problems])
            z = np.zeros(len(self.problems))
            return t, z.astype(np.int32), (z - 1).astype(np.int64)

        def get_state(self, k, stream=None):
            return self.problems[k]["state"]

        def set_state(self, k, planes, t, stream=None):
            self.problems[k].update(t=t, state=planes)

        def step(self, n, stream=None):
            for q in self.problems:
                q["t"] = min(q["t"] + n * DT, q["t_end"])
                q["steps"] += n

        def close(self):
            pass

    def fake_assign(batch, dmeshes, cfl, final_time, keep=None, stream=None):
        new = []
        for k, dm in enumerate(dmeshes):
            if keep[k] >= 0:
                carried = batch.problems[keep[k]]
                assert carried["dm"] is dm  # the same request's problem is carried
                new.append(carried)
            else:
                new.append({"t": None, "t_end": final_time[k], "dm": dm, "steps": 0})
        assigns.append((len(dmeshes), sum(dm.num_cells for dm in dmeshes)))
        batch.problems, batch.meshes = new, list(dmeshes)

    monkeypatch.setattr(H, "Batch", FakeBatch)
    monkeypatch.setattr(H, "DeviceMesh", FakeDeviceMesh)
    monkeypatch.setattr(H, "batch_assign_device", fake_assign)
    reqs = [serve.Request(k, 0.002 * k, side, "sod", t_end)
            for k, (side, t_end) in enumerate([(12, 0.05), (10, 0.2), (14, 0.1), (8, 0.05),
                                               (12, 0.3), (9, 0.08)])]
    p = serve.server_params()
    srv = serve.Server(p, max_cells=300, max_faces=10**6, max_vertices=10**6, max_problems=3,
                       steps_per_launch=2, build_threads=2)
    try:
        out = srv.run(reqs, time_limit=60.0)
    finally:
        srv.close()
    assert out["requests_done"] == len(reqs) and out["failed"] == 0
    assert out["reassignments"] == len(assigns) >= 3
    assert all(n <= 3 and cells <= 300 for n, cells in assigns)  # within every capacity
    for r in out["done"]:
        assert abs(r.t_final - r.t_end) <= 1e-12 * r.t_end  # ran to its own end time
        assert r.result is r.state0                       # and returned its own state
        assert r.admitted >= 0 and r.finished >= r.admitted
    # 6 requests, 832 cells in all, through a 300-cell batch: some had to wait for a slot
    assert any(r.admitted > min(q.finished for q in reqs) for r in reqs)
