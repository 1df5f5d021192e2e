"""The command-line driver (apps/hydro's executable, driver.h:163-450) on the
GPU: the reference's own regression flow -- input file + Exodus mesh in,
regression dump out, numdiff against the .std golden -- and a run whose mesh
comes from the input's box table."""
import os
import subprocess

import numpy as np
import pytest

import flecsale_gb300.hydro as H
from flecsale_gb300 import numdiff
from tests import _util as U
from tests.test_io import _write_exodus, golden_2d_text

pytestmark = pytest.mark.gpu
INPUTS = os.path.join(U.GOLDEN, "inputs")


def _run(args, cwd):
    r = subprocess.run([H.driver_path(), *args], capture_output=True, text=True, timeout=600,
                       cwd=cwd)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_cli_2d_regression(tmp_path):
    pytest.importorskip("scipy")
    mesh, z = U.golden_2d()
    a = mesh.arrays()
    g = str(tmp_path / "square_32x32.g")
    _write_exodus(g, a["vertex_coord"].T.copy(), a["cell_vertices"].reshape(-1, 4), "QUAD4")
    out = _run(["-f", os.path.join(INPUTS, "shock_box_2d.lua"), "-m", g,
                "--output_dir", str(tmp_path)], str(tmp_path))
    assert 'Using input file' in out and "after 20 steps." in out
    dump = tmp_path / "shock_box_2d-solution_rank000000.txt"
    rep = numdiff.compare_lines(golden_2d_text(), dump.read_text().splitlines(),
                                abs_tol=2e-14, check_text=True)
    assert rep.ok, rep.failures


def test_cli_3d_box_mesh_matches_library_run(tmp_path):
    _run(["-f", os.path.join(INPUTS, "shock_box_3d_box.lua"), "--output_dir", str(tmp_path)],
         str(tmp_path))
    got = (tmp_path / "shock_box_3d-solution_rank000000.txt").read_text()
    inp = H.Input(os.path.join(INPUTS, "shock_box_3d_box.lua"))
    p, max_steps, _ = inp.params(3)
    mesh = inp.mesh()
    state = inp.initial_state(mesh, p)
    dm, ds = H.DeviceMesh(mesh), H.DeviceState(3, mesh.num_cells)
    s = H.Solver(dm, p)
    ds.upload(state)
    s.reset(0.0)
    n = s.run(ds, max_steps)
    code, t, _ = s.status()
    assert code == 0 and n == 12
    ref = str(tmp_path / "ref.txt")
    H.write_dump(ref, mesh, ds.download(), t, n)
    assert got == open(ref).read()
    # the shock has moved: not the initial state any more
    assert "# Number iterations: 12" in got


def test_cli_mixed_precision_option(tmp_path):
    """--precision mixed --flux hllc: the dump read back is within relative L1
    1e-4 (density and total energy, the mixed form's bar) of a library run of
    the mixed form on the same input, and of the FP64 library run."""
    out = _run(["-f", os.path.join(INPUTS, "shock_box_3d_box.lua"), "--precision", "mixed",
                "--flux", "hllc", "--output_dir", str(tmp_path)], str(tmp_path))
    assert "after 12 steps." in out
    inp = H.Input(os.path.join(INPUTS, "shock_box_3d_box.lua"))
    p64, max_steps, _ = inp.params(3)
    mesh = inp.mesh()
    got, t_cli, n_cli = H.read_dump(str(tmp_path / "shock_box_3d-solution_rank000000.txt"), 3,
                                    mesh.num_cells, p64.gamma, p64.cv)
    assert n_cli == 12
    E = lambda s: s[0] * (s[4] + 0.5 * (s[1] ** 2 + s[2] ** 2 + s[3] ** 2))
    l1 = lambda a, b: np.abs(a - b).sum() / np.abs(b).sum()
    for precision in ("mixed", "fp64"):
        p = H.Params.from_buffer_copy(p64)  # the input file's settings, as the driver reads them
        p.flux_kind, p.precision = H.FLUX["hllc"], H.PRECISION[precision]
        state = inp.initial_state(mesh, p)
        dm, ds = H.DeviceMesh(mesh), H.DeviceState(3, mesh.num_cells)
        s = H.Solver(dm, p)
        ds.upload(state)
        s.reset(0.0)
        assert s.run(ds, max_steps) == 12
        code, t, _ = s.status()
        lib_run = ds.download()
        assert code == 0 and abs(t - t_cli) <= 1e-4 * t
        assert l1(got[0], lib_run[0]) <= 1e-4 and l1(E(got), E(lib_run)) <= 1e-4, precision
