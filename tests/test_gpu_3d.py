"""3D shock box on hexahedra (the 192^3 configuration at a quarter of the
resolution per axis): FP64 vs mixed after 100 steps.  Tolerance written out:
relative L1 of density and total energy <= 1e-4."""
import numpy as np
import pytest

import flecsale_gb300.hydro as H

pytestmark = pytest.mark.gpu


def test_3d_shock_box_mixed_vs_fp64():
    mesh = H.HostMesh.box(3, (48, 48, 48), [0, 0, 0], [1, 1, 1], 0.15, 2)
    kw = dict(flux="rusanov", cfl=0.3, final_time=1e9)
    s0 = H.initial_state("inner_cube", mesh, H.make_params(3, **kw))
    dm = H.DeviceMesh(mesh)
    res = {}
    for form in ("fp64", "mixed"):
        ds, sv = H.DeviceState(3, mesh.num_cells), H.Solver(dm, H.make_params(3, precision=form, **kw))
        ds.upload(s0)
        sv.reset(0.0)
        sv.run(ds, 100)
        assert sv.status()[0] == 0
        res[form] = ds.download()
    f, m = res["fp64"], res["mixed"]
    E = lambda s: s[0] * (s[4] + 0.5 * (s[1] ** 2 + s[2] ** 2 + s[3] ** 2))
    assert np.abs(m[0] - f[0]).sum() / np.abs(f[0]).sum() <= 1e-4
    assert np.abs(E(m) - E(f)).sum() / np.abs(E(f)).sum() <= 1e-4
    vol = mesh.arrays()["cell_volume"]
    assert abs(np.sum(m[0] * vol) - np.sum(s0[0] * vol)) / np.sum(s0[0] * vol) < 1e-12
