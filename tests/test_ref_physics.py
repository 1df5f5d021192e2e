"""The oracle's physics against the reference's own code.

oracle/_ref/libref_physics.so is the reference's flecsale/eqns/euler_eqns.h,
flecsale/eqns/flux.h and flecsale/eos/ideal_gas.h compiled unchanged
(oracle/ref_build.py).  Its outputs on seeded random states are committed in
tests/golden/ref_physics_vectors.npz (tests/golden/make_golden.py); where the
reference checkout exists the library is also called live on fresh inputs.
Every comparison is bitwise.
"""
import ctypes as C
import os

import numpy as np
import pytest

from tests import _util as U
from tests.golden.make_golden import physics_cases

dp = C.POINTER(C.c_double)


def _p(x):
    return np.ascontiguousarray(x).ctypes.data_as(dp)


def _oracle_flux(O, dim, kind, wl, wr, n):
    f = np.zeros(dim + 2)
    O.oracle_face_flux(dim, kind, _p(wl), _p(wr), _p(n), f.ctypes.data_as(dp))
    return f


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", [-1, 0, 1], ids=["wall", "hlle", "rusanov"])
def test_oracle_flux_matches_reference_vectors(oracle_lib, dim, kind):
    z = np.load(os.path.join(U.GOLDEN, "ref_physics_vectors.npz"))
    wl, wr, nrm, _ = physics_cases(dim, 64, 100 + dim)
    ref = z[f"flux_{dim}d_{kind}"]
    got = np.array([_oracle_flux(oracle_lib, dim, kind, wl[i], wr[i], nrm[i]) for i in range(len(wl))])
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_update_matches_reference_vectors(oracle_lib, dim):
    z = np.load(os.path.join(U.GOLDEN, "ref_physics_vectors.npz"))
    wl, _, _, du = physics_cases(dim, 64, 100 + dim)
    got = wl.copy()
    for i in range(len(got)):
        row = np.ascontiguousarray(got[i])
        oracle_lib.oracle_update_cell(dim, 1.4, 1.0, row.ctypes.data_as(dp), _p(du[i]))
        got[i] = row
    assert np.array_equal(got, z[f"update_{dim}d"], equal_nan=True)


def _ref_lib():
    from oracle import ref_build
    if not ref_build.available():
        pytest.skip("reference checkout not present")
    L = C.CDLL(ref_build.build())
    L.ref_face_flux.argtypes = [C.c_int32, C.c_int32, dp, dp, dp, dp]
    L.ref_update_cell.argtypes = [C.c_int32, C.c_double, C.c_double, dp, dp]
    L.ref_state_from_pressure.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, dp, dp, dp]
    return L


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_matches_live_reference(oracle_lib, dim):
    R = _ref_lib()
    wl, wr, nrm, du = physics_cases(dim, 500, 7 + dim)
    for kind in (-1, 0, 1):
        for i in range(len(wl)):
            fr = np.zeros(dim + 2)
            R.ref_face_flux(dim, kind, _p(wl[i]), _p(wr[i]), _p(nrm[i]), fr.ctypes.data_as(dp))
            assert np.array_equal(_oracle_flux(oracle_lib, dim, kind, wl[i], wr[i], nrm[i]), fr)
    for i in range(len(wl)):
        a, b = wl[i].copy(), wl[i].copy()
        R.ref_update_cell(dim, 1.4, 1.0, a.ctypes.data_as(dp), _p(du[i]))
        oracle_lib.oracle_update_cell(dim, 1.4, 1.0, b.ctypes.data_as(dp), _p(du[i]))
        assert np.array_equal(a, b, equal_nan=True)
    rng = np.random.default_rng(3)
    for _ in range(200):
        g, cv, d, p = rng.uniform(1.1, 3), rng.uniform(0.5, 2), rng.uniform(0.1, 3), rng.uniform(0.1, 3)
        e, T, a = C.c_double(), C.c_double(), C.c_double()
        R.ref_state_from_pressure(g, cv, d, p, C.byref(e), C.byref(T), C.byref(a))
        eo, To, ao = np.zeros(1), np.zeros(1), np.zeros(1)
        oracle_lib.oracle_state_from_pressure(1, g, cv, _p(np.array([d])), _p(np.array([p])),
                                              eo.ctypes.data_as(dp), To.ctypes.data_as(dp), ao.ctypes.data_as(dp))
        assert (e.value, T.value, a.value) == (eo[0], To[0], ao[0])
