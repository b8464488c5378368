"""Analytic solutions used as accuracy oracles -- TEST INFRASTRUCTURE ONLY.

* ``heat_series``: the insulated-rod cosine series the reference's accuracy test
  uses for the parabolic IC (SweptSource/Testing/testProcedure.py:63-82),
  restated in numpy.
* ``heat_periodic_mode``: the single decaying Fourier mode of the periodic
  heat problem (T = mean + A sin(2 pi x / L)), exactly for the FTCS scheme
  (amplification 1 - 4 Fo sin^2(pi/nx) per step) and for the PDE.
* ``sod``: the exact Riemann solution of the Sod shock tube.  The reference's
  test calls LANL ExactPack's ``Sod`` (testProcedure.py:16,84-96; not vendored,
  version not pinned); this is an independent restatement of the published
  exact solver (E. F. Toro, "Riemann Solvers and Numerical Methods for Fluid
  Dynamics", ch. 4: pressure function, Newton iteration for p*, wave sampling).
"""
from __future__ import annotations

import math

import numpy as np


def heat_series(t: float, divs: int, alpha: float = 8.418e-5, dx: float = 0.001, nterms: int = 5000) -> np.ndarray:
    """testProcedure.heat_exact: T = c0 - cout * sum_{n even} n^-2 e^{-alpha t (n pi/L)^2} cos(n pi x/L),
    L = divs*dx, x = linspace(0, L, divs), c0 = 50L/3, cout = 400L/pi^2, n = 2, 4, ..., 2 + 2*nterms."""
    L = divs * dx
    x = np.linspace(0.0, L, divs)
    n = 2.0 * np.arange(1, nterms + 2, dtype=np.float64)
    c0 = 50.0 * L / 3.0
    cout = 400.0 * L / np.pi ** 2
    h = np.zeros(divs)
    for nk in n:  # summed in the same order as the reference script
        h += 1.0 / nk ** 2 * np.exp(-alpha * t * (nk * np.pi / L) ** 2) * np.cos(nk * x * np.pi / L)
    return c0 - cout * h


def heat_periodic_mode(nsteps: int, nx: int, fourier: float, mean: float = 50.0, amp: float = 100.0,
                       discrete: bool = True, alpha: float = 8.418e-5, dx: float = 0.001,
                       fourier_two: float | None = None) -> np.ndarray:
    """Periodic heat, IC mean + amp sin(2 pi x/L), L = nx dx, after nsteps FTCS steps.
    discrete=True: the scheme's own exact answer -- per step the mean is
    multiplied by fo2 + 2 fo and the mode by fo2 + 2 fo cos(2 pi/nx), with
    fo2 = 1 - 2 fo unless the run's rounded value is given;
    discrete=False: the PDE's exp(-alpha (2 pi/L)^2 t), t = nsteps * Fo dx^2/alpha."""
    x = np.arange(nx) * dx
    L = nx * dx
    if discrete:
        fo2 = (1.0 - 2.0 * fourier) if fourier_two is None else fourier_two
        g0 = (fo2 + 2.0 * fourier) ** nsteps
        g = (fo2 + 2.0 * fourier * math.cos(2 * math.pi / nx)) ** nsteps
        return mean * g0 + amp * g * np.sin(2 * np.pi * x / L)
    t = nsteps * fourier * dx * dx / alpha
    g = math.exp(-alpha * (2 * math.pi / L) ** 2 * t)
    return mean + amp * g * np.sin(2 * np.pi * x / L)


def _pressure_function(p, rho, pk, ck, gamma):
    if p > pk:  # shock
        A = 2.0 / ((gamma + 1.0) * rho)
        B = (gamma - 1.0) / (gamma + 1.0) * pk
        f = (p - pk) * math.sqrt(A / (p + B))
        df = math.sqrt(A / (B + p)) * (1.0 - 0.5 * (p - pk) / (B + p))
    else:  # rarefaction
        pr = p / pk
        f = 2.0 * ck / (gamma - 1.0) * (pr ** ((gamma - 1.0) / (2.0 * gamma)) - 1.0)
        df = 1.0 / (rho * ck) * pr ** (-(gamma + 1.0) / (2.0 * gamma))
    return f, df


def sod_star(left=(1.0, 0.0, 1.0), right=(0.125, 0.0, 0.1), gamma: float = 1.4):
    """Star-region pressure and velocity (Toro 4.2-4.3, Newton-Raphson)."""
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = math.sqrt(gamma * pl / rl), math.sqrt(gamma * pr / rr)
    # two-rarefaction initial guess (Toro 4.46)
    z = (gamma - 1.0) / (2.0 * gamma)
    p = ((cl + cr - 0.5 * (gamma - 1.0) * (ur - ul)) / (cl / pl ** z + cr / pr ** z)) ** (1.0 / z)
    p = max(p, 1e-12)
    for _ in range(200):
        fl, dfl = _pressure_function(p, rl, pl, cl, gamma)
        fr, dfr = _pressure_function(p, rr, pr, cr, gamma)
        pn = p - (fl + fr + ur - ul) / (dfl + dfr)
        pn = max(pn, 1e-12)
        if abs(pn - p) / (0.5 * (pn + p)) < 1e-15:
            p = pn
            break
        p = pn
    fl, _ = _pressure_function(p, rl, pl, cl, gamma)
    fr, _ = _pressure_function(p, rr, pr, cr, gamma)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sod(x: np.ndarray, t: float, x0: float = 0.5, left=(1.0, 0.0, 1.0), right=(0.125, 0.0, 0.1),
        gamma: float = 1.4) -> dict:
    """Exact Sod solution at positions x and time t: density, velocity, pressure,
    energy (specific internal energy p/((gamma-1) rho), the reference .dat's 'Energy')."""
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = math.sqrt(gamma * pl / rl), math.sqrt(gamma * pr / rr)
    ps, us = sod_star(left, right, gamma)
    g1 = (gamma - 1.0) / (gamma + 1.0)
    x = np.asarray(x, dtype=np.float64)
    rho = np.empty_like(x)
    u = np.empty_like(x)
    p = np.empty_like(x)
    for i, xi in enumerate(x):
        s = (xi - x0) / t if t > 0 else (math.inf if xi >= x0 else -math.inf)
        if s <= us:  # left of contact
            if ps > pl:  # left shock
                sl = ul - cl * math.sqrt((gamma + 1) / (2 * gamma) * ps / pl + (gamma - 1) / (2 * gamma))
                if s <= sl:
                    w = (rl, ul, pl)
                else:
                    w = (rl * (ps / pl + g1) / (g1 * ps / pl + 1.0), us, ps)
            else:  # left rarefaction
                shl = ul - cl
                if s <= shl:
                    w = (rl, ul, pl)
                else:
                    cml = cl * (ps / pl) ** ((gamma - 1) / (2 * gamma))
                    stl = us - cml
                    if s > stl:
                        w = (rl * (ps / pl) ** (1.0 / gamma), us, ps)
                    else:
                        uu = 2.0 / (gamma + 1) * (cl + 0.5 * (gamma - 1) * ul + s)
                        c = 2.0 / (gamma + 1) * (cl + 0.5 * (gamma - 1) * (ul - s))
                        w = (rl * (c / cl) ** (2.0 / (gamma - 1)), uu, pl * (c / cl) ** (2.0 * gamma / (gamma - 1)))
        else:  # right of contact
            if ps > pr:  # right shock
                sr = ur + cr * math.sqrt((gamma + 1) / (2 * gamma) * ps / pr + (gamma - 1) / (2 * gamma))
                if s >= sr:
                    w = (rr, ur, pr)
                else:
                    w = (rr * (ps / pr + g1) / (g1 * ps / pr + 1.0), us, ps)
            else:  # right rarefaction
                shr = ur + cr
                if s >= shr:
                    w = (rr, ur, pr)
                else:
                    cmr = cr * (ps / pr) ** ((gamma - 1) / (2 * gamma))
                    str_ = us + cmr
                    if s <= str_:
                        w = (rr * (ps / pr) ** (1.0 / gamma), us, ps)
                    else:
                        uu = 2.0 / (gamma + 1) * (-cr + 0.5 * (gamma - 1) * ur + s)
                        c = 2.0 / (gamma + 1) * (cr - 0.5 * (gamma - 1) * (ur - s))
                        w = (rr * (c / cr) ** (2.0 / (gamma - 1)), uu, pr * (c / cr) ** (2.0 * gamma / (gamma - 1)))
        rho[i], u[i], p[i] = w
    return {"density": rho, "velocity": u, "pressure": p, "energy": p / ((gamma - 1.0) * rho)}


def sod_cell_centres(divs: int) -> np.ndarray:
    """Interior cell centres of the reference's Euler grid (testProcedure.py:84-96):
    dx = 1/(divs-2), x = dx/2, 3dx/2, ..., 1 - dx/2."""
    dx = 1.0 / float(divs - 2)
    return (np.arange(divs - 2) + 0.5) * dx
