"""The C-ABI library loads and exports every function include/flecsale_gb300.h
declares (no GPU needed: nothing here launches a kernel)."""
import ctypes as C
import os
import re

import numpy as np

import flecsale_gb300.hydro as H

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_functions():
    names = set()
    for fn in os.listdir(HEADER):
        if fn.endswith(".h"):
            text = open(os.path.join(HEADER, fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(fvh_[a-z0-9_]+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(fvh):
    names = declared_functions()
    assert len(names) > 30
    L = fvh.lib()
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_abi_basics(fvh):
    L = fvh.lib()
    assert L.fvh_abi_version() == 1
    assert L.fvh_status_string(4) == b"Negative density or internal energy encountered!"
    assert L.fvh_status_string(3) == b"infinite delta t"
    p = fvh.Params()
    L.fvh_params_default(C.byref(p), 2)
    assert (p.flux_kind, p.limiter, p.order, p.recon_swap_ep) == (0, 0, 2, 1)
    assert (p.gamma, p.cv, p.cfl, p.final_time) == (1.4, 1.0, 0.5, 0.2)
    code, cell = C.c_int32(), C.c_int64()
    L.fvh_status_decode(C.c_uint64((123 << 8) | 4), C.byref(code), C.byref(cell))
    assert (code.value, cell.value) == (4, 123)
    L.fvh_status_decode(C.c_uint64(H.STATUS_CLEAR), C.byref(code), C.byref(cell))
    assert (code.value, cell.value) == (0, -1)


def test_argument_errors_without_gpu(fvh):
    """Argument checks happen before any device call."""
    L = fvh.lib()
    m = fvh.HostMesh.box(2, [4, 4], [0, 0], [1, 1])
    p = fvh.make_params(2)
    bad = fvh.make_params(3)
    s = fvh.StateView()
    assert L.fvh_evaluate_gradients(C.byref(m.view), C.byref(s), None, C.byref(p), None) == H.ERR_INVALID_ARGUMENT
    st = np.zeros((8, m.num_cells))
    sv = H.host_state_view(st, 2)
    g = fvh.GradientView()
    assert L.fvh_evaluate_gradients(C.byref(m.view), C.byref(sv), C.byref(g), C.byref(bad), None) == H.ERR_INVALID_ARGUMENT
    h = C.c_void_p()
    assert L.fvh_host_mesh_box(4, None, None, None, 0.0, 0, C.byref(h)) == H.ERR_INVALID_ARGUMENT
    assert L.fvh_time_step_workspace_bytes(10**6) == 8 * 1216


def test_solver_and_batch_entry_points_reject_null_handles(fvh):
    """The solver/batch entry points beyond the reference's tasks check their
    handles and counts before any device call (no GPU needed)."""
    L = fvh.lib()
    EI = H.ERR_INVALID_ARGUMENT
    sv = fvh.StateView()
    i32, dbl = C.c_int32(), C.c_double()
    assert L.fvh_solver_set_shape(None, 128, 1, 1) == EI
    assert L.fvh_solver_autotune(None, C.byref(sv), 3, C.byref(i32), C.byref(i32),
                                 C.byref(i32), C.byref(dbl), None) == EI
    assert L.fvh_solver_advance_host(None, C.byref(sv), None, 1, C.byref(dbl), None) == EI
    assert L.fvh_solver_launches_per_run(None, 10) == 0
    assert L.fvh_debug_split(None, -1, None, None, None, None, None) == EI
    assert L.fvh_batch_step(None, 1, None) == EI


def test_missing_library_fails_loudly_without_a_fallback(tmp_path):
    """With the shared library absent and no CUDA compiler to build it, the
    binding raises instead of falling back to any other implementation (in a
    child process, so the library this session loaded stays untouched)."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = f"""
import shutil
import flecsale_gb300._build as B
import flecsale_gb300.hydro as H
B.LIB = {str(tmp_path / 'absent' / 'libflecsale_gb300.so')!r}
shutil.which = lambda name, *a, **k: None
B._nvcc = lambda: (_ for _ in ()).throw(RuntimeError("nvcc not found: the CUDA toolkit is required"))
try:
    H.lib()
except RuntimeError as e:
    print("raised", e)
else:
    print("loaded")
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120,
                       cwd=root, env=dict(os.environ, PYTHONPATH=root))
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.startswith("raised") and "nvcc not found" in r.stdout, r.stdout
