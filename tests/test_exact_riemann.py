"""The oracle's Riemann fluxes against the exact solution of the Riemann
problem (CPU only).

HLLC has no counterpart in the reference, and the reference's own tests never
run HLLE or Rusanov on a problem with a known answer, so these tests check the
restated schemes against the exact solution of the 1D Riemann problem for an
ideal gas: the iterative star-pressure solve and self-similar sampling of
E. F. Toro, "Riemann Solvers and Numerical Methods for Fluid Dynamics", 3rd ed.,
ch. 4 (written here from the method, in numpy).  The workload is the CPU-
runnable Sod case: 100 x 10 quads on [0,1] x [0,0.1], walls, gamma 1.4, CFL 0.5,
first order, run to t = 0.2; finer meshes check convergence.  The GPU FP64 path
is bitwise equal to the oracle, so the same bounds hold for it.
"""
import numpy as np
import pytest

import flecsale_gb300.hydro as H
from tests import _util as U

SOD_L, SOD_R, GAMMA = (1.0, 0.0, 1.0), (0.125, 0.0, 0.1), 1.4


def _pressure_function(p, rho, pk, gamma):
    """f_K(p) and its derivative for one side (shock if p > p_K, else rarefaction)."""
    a = np.sqrt(gamma * pk / rho)
    if p > pk:
        A, B = 2.0 / ((gamma + 1.0) * rho), (gamma - 1.0) / (gamma + 1.0) * pk
        q = np.sqrt(A / (p + B))
        return (p - pk) * q, q * (1.0 - 0.5 * (p - pk) / (B + p))
    r = (p / pk) ** ((gamma - 1.0) / (2.0 * gamma))
    return 2.0 * a / (gamma - 1.0) * (r - 1.0), r / (rho * a) * (pk / p)


def star_state(left, right, gamma):
    """(p*, u*, rho*_L, rho*_R) by Newton iteration on f_L + f_R + du = 0."""
    (rl, ul, pl), (rr, ur, pr) = left, right
    p = max(1e-12, 0.5 * (pl + pr))
    for _ in range(100):
        fl, dl = _pressure_function(p, rl, pl, gamma)
        fr, dr = _pressure_function(p, rr, pr, gamma)
        step = (fl + fr + ur - ul) / (dl + dr)
        p_new = max(1e-12, p - step)
        if abs(p_new - p) <= 1e-15 * (p_new + p):
            p = p_new
            break
        p = p_new
    fl, _ = _pressure_function(p, rl, pl, gamma)
    fr, _ = _pressure_function(p, rr, pr, gamma)
    u = 0.5 * (ul + ur) + 0.5 * (fr - fl)
    g = (gamma - 1.0) / (gamma + 1.0)

    def rho_star(rho, pk):
        if p > pk:
            return rho * (p / pk + g) / (g * p / pk + 1.0)
        return rho * (p / pk) ** (1.0 / gamma)

    return p, u, rho_star(rl, pl), rho_star(rr, pr)


def exact_riemann(left, right, gamma, s):
    """(rho, u, p) of the exact solution at the similarity coordinates s = x/t."""
    s = np.asarray(s, np.float64)
    p_s, u_s, rls, rrs = star_state(left, right, gamma)
    out = np.empty((3,) + s.shape)
    for side, (rho, u, pk), rho_s, sign in ((0, left, rls, -1.0), (1, right, rrs, 1.0)):
        on_side = s <= u_s if side == 0 else s > u_s
        a = np.sqrt(gamma * pk / rho)
        # work in the frame where this side's waves move in the -sign direction
        xi = sign * s
        un, usn = sign * u, sign * u_s
        if p_s > pk:  # shock
            ws = un + a * np.sqrt((gamma + 1) / (2 * gamma) * p_s / pk + (gamma - 1) / (2 * gamma))
            far = xi >= ws
            vals = [np.where(far, rho, rho_s), np.where(far, u, u_s), np.where(far, pk, p_s)]
        else:  # rarefaction
            a_s = a * (p_s / pk) ** ((gamma - 1) / (2 * gamma))
            head, tail = un + a, usn + a_s
            c = 2.0 / (gamma + 1) * (a - (gamma - 1) / 2 * (un - xi))
            fan_u = sign * 2.0 / (gamma + 1) * (-a + (gamma - 1) / 2 * un + xi)
            fan_rho = rho * (c / a) ** (2 / (gamma - 1))
            fan_p = pk * (c / a) ** (2 * gamma / (gamma - 1))
            vals = [np.where(xi >= head, rho, np.where(xi <= tail, rho_s, fan_rho)),
                    np.where(xi >= head, u, np.where(xi <= tail, u_s, fan_u)),
                    np.where(xi >= head, pk, np.where(xi <= tail, p_s, fan_p))]
        for q in range(3):
            out[q] = np.where(on_side, vals[q], out[q]) if side else np.where(on_side, vals[q], 0.0)
    return out


def _run_sod(O, n, ny, flux, order):
    """Oracle run of Sod on n x ny quads of height h (so cells are square), to t = 0.2."""
    mesh = H.HostMesh.box(2, (n, ny), [0, 0], [1, ny / n])
    p = H.make_params(2, flux=flux, order=order, swap=False, cfl=0.5, final_time=0.2)
    state = H.initial_state("sod", mesh, p)
    mass0 = float((state[0] * mesh.arrays()["cell_volume"]).sum())
    st, t, steps = U.oracle_run(O, mesh, state, p, 100000, stop_at_final=True)
    assert st == 0 and abs(t - 0.2) <= 1e-14 and steps > 0
    x = mesh.arrays()["cell_centroid"][0].copy()
    mass = float((state[0] * mesh.arrays()["cell_volume"]).sum())
    assert abs(mass - mass0) <= 1e-13 * mass0  # walls: mass is conserved
    return x, state, t


def _l1(x, rho, t, lo=0.0, hi=1.0):
    exact = exact_riemann(SOD_L, SOD_R, GAMMA, (x - 0.5) / t)[0]
    w = (x >= lo) & (x <= hi)
    return float(np.abs(rho - exact)[w].mean() * (hi - lo))


def test_exact_solver_reproduces_the_published_sod_star_state():
    """Toro, Table 4.3, test 1: p* = 0.30313, u* = 0.92745, rho*_L = 0.42632,
    rho*_R = 0.26557 (5 significant digits)."""
    p, u, rl, rr = star_state(SOD_L, SOD_R, GAMMA)
    for got, want in ((p, 0.30313), (u, 0.92745), (rl, 0.42632), (rr, 0.26557)):
        assert abs(got - want) <= 5e-6, (got, want)
    rho, vel, pres = exact_riemann(SOD_L, SOD_R, GAMMA, np.array([-2.0, 0.0, 0.5, 1.5, 2.0]))
    assert rho[0] == 1.0 and pres[0] == 1.0 and rho[-1] == 0.125 and pres[-1] == 0.1
    assert abs(pres[2] - p) < 1e-12 and abs(vel[3] - u) < 1e-12 and abs(rho[3] - rr) < 1e-12


def test_sod_first_order_hllc_against_the_exact_solution(fvh, oracle_lib):
    """The CPU-runnable case exactly: 100 x 10 quads on [0,1] x [0,0.1],
    first-order HLLC, CFL 0.5, to t = 0.2.  The 1D solution stays 1D (every row
    of cells the same, no y velocity) and lies within first-order distance of
    the exact solution."""
    x, s, t = _run_sod(oracle_lib, 100, 10, "hllc", 1)
    rows = s.reshape(s.shape[0], 10, 100)
    assert np.abs(rows - rows[:, :1]).max() <= 1e-13
    assert np.abs(s[2]).max() <= 1e-13
    l1 = _l1(x, s[0], t)
    assert 0.005 < l1 <= 0.021, l1


def test_schemes_converge_to_the_exact_solution(fvh, oracle_lib):
    """First order: the L1 density error falls by at least 1.4x per mesh
    doubling for each flux, and the fluxes rank by how little they diffuse
    (HLLC < HLLE < Rusanov), with HLLC sharper than HLLE at the contact.
    Second order (MUSCL with the Barth-Jespersen limiter) is at least 3x
    closer than first order."""
    err = {}
    for flux in ("hllc", "hlle", "rusanov"):
        for n in (100, 200, 400):
            x, s, t = _run_sod(oracle_lib, n, 4, flux, 1)
            err[flux, n] = _l1(x, s[0], t)
            if n == 100:
                err[flux, "contact"] = _l1(x, s[0], t, 0.62, 0.75)
        assert err[flux, 100] / err[flux, 200] >= 1.4 and err[flux, 200] / err[flux, 400] >= 1.4, err
    assert err["hllc", 100] < err["hlle", 100] < err["rusanov", 100], err
    assert err["hllc", "contact"] < err["hlle", "contact"], err
    x, s, t = _run_sod(oracle_lib, 100, 4, "hllc", 2)
    second = _l1(x, s[0], t)
    assert second * 3 <= err["hllc", 100] and second <= 0.005, (second, err["hllc", 100])
