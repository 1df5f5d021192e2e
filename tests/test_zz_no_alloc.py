"""fvh_evaluate_time_step_noalloc, the time-step entry point that allocates
nothing.

It is for callers that cannot allocate device memory: a task runtime that owns
all device memory and hands a task only its field buffers, or a hot loop that
must not pay cudaMalloc's implicit synchronisation.  Its scratch (the per-block
partial maxima) is a fixed 64 KiB array inside the library, shared by all calls.

The test calls it through the C ABI twice in a row, on two different states,
and checks each result against fvh_evaluate_time_step with a caller workspace
and against the oracle's evaluate_time_step.  The dt kernels are the bit-exact
FP64 ones, so the tolerance is exact equality, as in the other dt parity tests.
The 640x512 case needs more blocks (1,280) than fvh_evaluate_time_step launches
(1,216, each striding over more cells), so the two entry points split the cells
differently there.  This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import flecsale_gb300.hydro as H
from tests import _util as U

pytestmark = pytest.mark.gpu


def _dt_with_workspace(torch, L, mesh_view, sv, p, scal, status):
    nb = L.fvh_time_step_workspace_bytes(mesh_view.num_cells)
    ws = torch.zeros(nb // 8 + 1, dtype=torch.float64, device="cuda")
    H.check(L.fvh_evaluate_time_step(C.byref(mesh_view), C.byref(sv), C.byref(p), scal.data_ptr(),
                                     scal.data_ptr() + 8, ws.data_ptr(), nb, status.data_ptr(), None))
    torch.cuda.synchronize()
    return float(scal[1].item()), int(status.item())


def _dt_noalloc(torch, L, mesh_view, sv, p, scal, status):
    H.check(L.fvh_evaluate_time_step_noalloc(C.byref(mesh_view), C.byref(sv), C.byref(p), scal.data_ptr(),
                                             scal.data_ptr() + 8, status.data_ptr(), None))
    torch.cuda.synchronize()
    return float(scal[1].item()), int(status.item())


@pytest.mark.parametrize("dim,n", [(2, (300, 200)), (2, (640, 512)), (3, (30, 24, 20))])
def test_noalloc_time_step_matches_workspace_version(cuda, dim, n):
    torch = cuda
    L = H.lib()
    O = __import__("oracle").load()
    if dim == 2:
        mesh = H.HostMesh.box(2, n, [0, 0], [1, 1], 0.2, 4)
        p = H.make_params(2, flux="hllc", cfl=0.4, boundary="outflow")
        problems = ("four_quadrant", "kelvin_helmholtz")
    else:
        mesh = H.HostMesh.box(3, n, [0, 0, 0], [1, 1, 1], 0.15, 4)
        p = H.make_params(3, flux="rusanov", cfl=0.3)
        problems = ("inner_cube", "kelvin_helmholtz")
    dmesh = H.DeviceMesh(mesh)
    for call, prob in enumerate(problems):  # two calls in a row, different states
        state = H.initial_state(prob, mesh, p, seed=call)
        ds = torch.tensor(state, device="cuda")
        sv = U.device_state_view(ds, dim)
        scal = torch.tensor([0.01, 0.0], dtype=torch.float64, device="cuda")
        status = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        dt_ref, st_ref = _dt_with_workspace(torch, L, dmesh.view, sv, p, scal, status)
        scal[1] = -1.0
        dt_new, st_new = _dt_noalloc(torch, L, dmesh.view, sv, p, scal, status)
        assert st_ref == -1 and st_new == -1
        assert dt_new == dt_ref and dt_new > 0
        st_o, dt_o = U.oracle_time_step(O, mesh, state, p, 0.01)
        assert st_o == 0 and dt_new == dt_o


def test_noalloc_rejects_meshes_beyond_capacity(cuda):
    """More cells than the fixed array covers: FVH_ERR_CAPACITY, nothing launched."""
    torch = cuda
    L = H.lib()
    cap = L.fvh_time_step_noalloc_max_cells()
    assert cap == 2097152
    mesh = H.HostMesh.box(2, (16, 16), [0, 0], [1, 1], 0.0, 0)
    dmesh = H.DeviceMesh(mesh)
    view = H.MeshView.from_buffer_copy(dmesh.view)
    view.num_cells = cap + 1
    p = H.make_params(2)
    ds = torch.zeros((7, mesh.num_cells), dtype=torch.float64, device="cuda")
    scal = torch.zeros(2, dtype=torch.float64, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    rc = L.fvh_evaluate_time_step_noalloc(C.byref(view), C.byref(U.device_state_view(ds, 2)), C.byref(p),
                                          scal.data_ptr(), scal.data_ptr() + 8, status.data_ptr(), None)
    assert rc == H.ERR_CAPACITY
    torch.cuda.synchronize()
    assert int(status.item()) == -1
    assert np.array_equal(scal.cpu().numpy(), [0.0, 0.0])
