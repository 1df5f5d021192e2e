"""Unit properties of the oracle's Riemann fluxes that no reference test
checks (CPU only): consistency F(w, w, n) = f(w).n, rotational invariance,
conservation under swapping the sides, the wall flux, and HLLC's exact
resolution of contact discontinuities (which HLLE and Rusanov smear).  The GPU
FP64 kernels compute these fluxes bitwise like the oracle."""
import ctypes as C

import numpy as np
import pytest

from tests import _util as U  # noqa: F401  (oracle_lib fixture lives in conftest)

dp = C.POINTER(C.c_double)
GAMMA, CV = 1.4, 1.0
KINDS = {"hlle": 0, "rusanov": 1, "hllc": 2}


def _w(dim, rho, v, p):
    """Primitive record (d, v[dim], p, e, T, a) of an ideal gas."""
    e = p / (rho * (GAMMA - 1.0))
    return np.array([rho, *v[:dim], p, e, e / CV, np.sqrt(GAMMA * (GAMMA - 1.0) * e)])


def _flux(O, dim, kind, wl, wr, n):
    f = np.zeros(dim + 2)
    O.oracle_face_flux(dim, kind, np.ascontiguousarray(wl).ctypes.data_as(dp),
                       np.ascontiguousarray(wr).ctypes.data_as(dp),
                       np.ascontiguousarray(n, np.float64).ctypes.data_as(dp), f.ctypes.data_as(dp))
    return f


def _physical(dim, w, n):
    rho, v, p, e = w[0], w[1:1 + dim], w[1 + dim], w[2 + dim]
    vn = float(v @ n)
    E = rho * (e + 0.5 * float(v @ v))
    return np.array([rho * vn, *(rho * v * vn + p * n), (E + p) * vn])


def _states(dim, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = rng.normal(size=dim)
        n /= np.linalg.norm(n)
        wl = _w(dim, rng.uniform(0.1, 3), rng.normal(size=dim), rng.uniform(0.05, 3))
        wr = _w(dim, rng.uniform(0.1, 3), rng.normal(size=dim), rng.uniform(0.05, 3))
        out.append((wl, wr, n))
    return out


def _rotation(dim, rng):
    q, r = np.linalg.qr(rng.normal(size=(dim, dim)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def _rotate(dim, w, R):
    out = w.copy()
    out[1:1 + dim] = R @ w[1:1 + dim]
    return out


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", sorted(KINDS))
def test_consistency(oracle_lib, dim, kind):
    """Equal states on both sides give the physical flux."""
    for wl, _, n in _states(dim, 50, 1 + dim):
        f = _flux(oracle_lib, dim, KINDS[kind], wl, wl, n)
        ref = _physical(dim, wl, n)
        assert np.allclose(f, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max()), (f, ref)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", sorted(KINDS))
def test_rotational_invariance(oracle_lib, dim, kind):
    """Rotating both states and the normal rotates the momentum flux and
    leaves the mass and energy fluxes unchanged."""
    rng = np.random.default_rng(20 + dim)
    for wl, wr, n in _states(dim, 50, 3 + dim):
        R = _rotation(dim, rng)
        f = _flux(oracle_lib, dim, KINDS[kind], wl, wr, n)
        g = _flux(oracle_lib, dim, KINDS[kind], _rotate(dim, wl, R), _rotate(dim, wr, R), R @ n)
        expect = np.array([f[0], *(R @ f[1:1 + dim]), f[1 + dim]])
        scale = np.abs(f).max() + 1.0
        assert np.abs(g - expect).max() <= 1e-13 * scale, (g, expect)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", sorted(KINDS))
def test_conservation_under_side_swap(oracle_lib, dim, kind):
    """The flux leaving one cell enters the other: F(wl, wr, n) = -F(wr, wl, -n)."""
    for wl, wr, n in _states(dim, 50, 5 + dim):
        f = _flux(oracle_lib, dim, KINDS[kind], wl, wr, n)
        g = _flux(oracle_lib, dim, KINDS[kind], wr, wl, -n)
        assert np.abs(f + g).max() <= 1e-13 * (np.abs(f).max() + 1.0), (f, g)


@pytest.mark.parametrize("dim", [2, 3])
def test_wall_flux(oracle_lib, dim):
    """Reflecting wall: no mass or energy crosses, momentum gets p n."""
    for wl, _, n in _states(dim, 20, 7 + dim):
        f = _flux(oracle_lib, dim, -1, wl, wl, n)
        assert f[0] == 0.0 and f[-1] == 0.0
        assert np.allclose(f[1:1 + dim], wl[1 + dim] * n, rtol=1e-15, atol=0)


@pytest.mark.parametrize("dim", [2, 3])
def test_hllc_resolves_contacts_exactly(oracle_lib, dim):
    """A contact (equal pressure and normal velocity, any density jump and
    any tangential velocities) gives the upwind side's physical flux with HLLC:
    a stationary contact carries no mass; HLLE and Rusanov diffuse both."""
    rng = np.random.default_rng(31 + dim)
    for un in (0.0, 0.4, -0.7):
        n = rng.normal(size=dim)
        n /= np.linalg.norm(n)
        t = rng.normal(size=dim)
        t -= (t @ n) * n
        wl = _w(dim, 1.0, un * n + 0.3 * t, 0.8)
        wr = _w(dim, 0.2, un * n - 0.5 * t, 0.8)
        up = wl if un >= 0 else wr
        f = _flux(oracle_lib, dim, KINDS["hllc"], wl, wr, n)
        ref = _physical(dim, up, n)
        assert np.abs(f - ref).max() <= 1e-14 * (np.abs(ref).max() + 1.0), (un, f, ref)
        if un == 0.0:
            assert abs(f[0]) <= 1e-15
        for kind in ("hlle", "rusanov"):
            g = _flux(oracle_lib, dim, KINDS[kind], wl, wr, n)
            assert abs(g[0] - ref[0]) > 1e-2, (kind, un, g, ref)
