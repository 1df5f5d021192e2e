"""The reference's regression tests, run on the GPU path: run the 2D shock box
(apps/hydro/2d) and the 3D shock box (apps/hydro/3d) through the C ABI, write
the dump of apps/hydro/tasks.h:771-849, and diff it with numdiff semantics
against the golden (see test_io.py for why the dump diff uses 2e-14)."""
import numpy as np
import pytest

import flecsale_gb300.hydro as H
from flecsale_gb300 import numdiff
from tests import _util as U
from tests.test_io import golden_2d_text

pytestmark = pytest.mark.gpu


def _run(mesh, p, nsteps):
    state = H.initial_state("shock_box", mesh, p)
    dm, ds = H.DeviceMesh(mesh), H.DeviceState(mesh.dim, mesh.num_cells)
    s = H.Solver(dm, p)
    ds.upload(state)
    s.reset(0.0)
    n = s.run(ds, nsteps)
    code, t, _ = s.status()
    assert code == 0
    return ds.download(), t, n


def test_gpu_dump_2d_regression(tmp_path):
    mesh, z = U.golden_2d()
    out, t, n = _run(mesh, H.make_params(2), 20)
    path = str(tmp_path / "shock_box_2d-solution_rank000000.txt")
    H.write_dump(path, mesh, out, t, n)
    rep = numdiff.compare_lines(golden_2d_text(), open(path).read().splitlines(),
                                abs_tol=2e-14, check_text=True)
    assert rep.ok, rep.failures


def test_gpu_dump_3d_regression(tmp_path):
    mesh, z = U.golden_3d()
    out, t, n = _run(mesh, H.make_params(3, cfl=1.0 / 3.0), 12)
    path = str(tmp_path / "shock_box_3d-solution_rank000000.txt")
    H.write_dump(path, mesh, out, t, n)
    lines = open(path).read().splitlines()
    assert lines[0] == f"# Solution time: {float(z['soln_time']):.14e}"
    assert lines[1] == "# Number iterations: 12"
    assert lines[4].startswith("# local_id global_id centroid(0) centroid(1) centroid(2) density")
    cells = np.array([[float(x) for x in l.split()] for l in lines[5:5 + 8000]])
    assert np.all(np.abs(cells[:, 5] - 1.0) <= 1e-14) and np.all(np.abs(cells[:, 6] - 2.5) <= 1e-14)
    assert np.all(np.abs(cells[:, 8:11]) <= 1e-14)
