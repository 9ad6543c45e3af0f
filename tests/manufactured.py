"""Analytic fields for the reference's accuracy checks, restated as tests.

The reference checks its sphere operators with three closed-form problems
(examples/test_slaplace.cpp:25-199 with scripts/test_slaplace.lua:25-54;
examples/test_barvortex.cpp:57-105, 216-242, 488-559 with
scripts/test_barvortex.lua:28-42 and scripts/test_jacobian.lua:28-33).  The
fields are the same; their derivatives are worked out here (no expression is
taken from the reference's sources) and checked by finite differences in
tests/test_manufactured.py.

Coordinates: phi = latitude, lam = longitude (the reference's zone-0 chart,
x = phi, y = lam).  On the unit sphere
    Laplacian f = f_phiphi - tan(phi) f_phi + f_lamlam / cos(phi)^2,
    J(u, v)     = (u_lam v_phi - u_phi v_lam) / cos(phi)   (src/sjacobian.cpp:410).
"""
from __future__ import annotations

import numpy as np


# ------------------------------------------------------------ Laplace --
def slaplace_u(phi, lam):
    """The Laplace test field 0.5 (x - 1)^2 + (x - z)^2 + 2 (z - 3)^2 with
    x = cos(phi) cos(lam), z = sin(phi) (the point's Cartesian coordinates)."""
    x = np.cos(phi) * np.cos(lam)
    z = np.sin(phi)
    return 0.5 * (x - 1.0) ** 2 + (x - z) ** 2 + 2.0 * (z - 3.0) ** 2


def slaplace_lapl(phi, lam):
    """Its spherical Laplacian.  For F(x, y, z) restricted to the unit
    sphere, Laplacian_S F = Laplacian F - F_rr - 2 F_r at r = 1 (F_r = p . grad
    F, F_rr = p^T Hess(F) p).  F = 1.5 x^2 - 2 x z + 3 z^2 - x - 12 z + 18.5:
    Laplacian F = 9, F_rr = 3 x^2 - 4 x z + 6 z^2, F_r = F_rr - x - 12 z, so
    Laplacian_S F = 9 - 9 x^2 + 12 x z - 18 z^2 + 2 x + 24 z."""
    x = np.cos(phi) * np.cos(lam)
    z = np.sin(phi)
    return 9.0 - 9.0 * x * x + 12.0 * x * z - 18.0 * z * z + 2.0 * x + 24.0 * z


# ----------------------------------------------------------- Jacobian --
def jac_f1(phi, lam):
    return np.sin(phi) * np.sin(lam)


def jac_f2(phi, lam):
    return np.cos(phi) * np.cos(lam)


def jac_exact(phi, lam):
    """J(sin phi sin lam, cos phi cos lam) =
    (-sin^2 phi cos^2 lam + cos^2 phi sin^2 lam) / cos phi."""
    c, s = np.cos(phi), np.sin(phi)
    return (-s * s * np.cos(lam) ** 2 + c * c * np.sin(lam) ** 2) / c


# --------------------------------------------------------- barvortex --
# stream function psi = g(phi) sin(lam + t), g = phi cos^4 phi; vorticity
# omega = Laplacian psi = w(phi) sin(lam + t) with w = g'' - tan g' - g / cos^2.
def _g(phi):
    c, s = np.cos(phi), np.sin(phi)
    return phi * c ** 4, c ** 4 - 4.0 * phi * c ** 3 * s


def _w(phi):
    """w, w', w'' (derivatives in phi), with c = cos, s = sin:
    w   = -9 c^3 s + 15 phi c^2 - 20 phi c^4
    w'  = 27 c^2 s^2 - 29 c^4 + 15 c^2 - 30 phi c s + 80 phi c^3 s
    w'' = -54 c s^3 + 250 c^3 s - 60 c s - 30 phi c^2 + 30 phi s^2 - 240 phi c^2 s^2 + 80 phi c^4"""
    c, s = np.cos(phi), np.sin(phi)
    w = -9.0 * c ** 3 * s + 15.0 * phi * c ** 2 - 20.0 * phi * c ** 4
    w1 = 27.0 * c * c * s * s - 29.0 * c ** 4 + 15.0 * c * c - 30.0 * phi * c * s + 80.0 * phi * c ** 3 * s
    w2 = (-54.0 * c * s ** 3 + 250.0 * c ** 3 * s - 60.0 * c * s - 30.0 * phi * c * c + 30.0 * phi * s * s
          - 240.0 * phi * c * c * s * s + 80.0 * phi * c ** 4)
    return w, w1, w2


def bv_psi(phi, lam, t):
    """The exact solution (stream function) at time t."""
    return _g(phi)[0] * np.sin(lam + t)


def bv_omega(phi, lam, t):
    return _w(phi)[0] * np.sin(lam + t)


def bv_forcing(phi, lam, t, sigma, mu):
    """f such that psi solves d(Lap psi)/dt + J(psi, Lap psi) + sigma Lap psi
    - mu Lap^2 psi = f with k1 = k2 = 1 and no Coriolis term (l + h = 0):
    f = w C + C S (g w' - g' w) / cos + sigma w S - mu (w'' - tan w' - w / cos^2) S,
    S = sin(lam + t), C = cos(lam + t).  Every term stays finite at the mesh's
    poles (cos(+-pi/2) rounds to 6e-17, and the quotients have removable
    singularities there)."""
    g, g1 = _g(phi)
    w, w1, w2 = _w(phi)
    c = np.cos(phi)
    S, C = np.sin(lam + t), np.cos(lam + t)
    with np.errstate(divide="ignore", invalid="ignore"):
        jac = C * S * (g * w1 - g1 * w) / c
        lap_w = w2 - np.tan(phi) * w1 - w / (c * c)
        return w * C + jac + sigma * w * S - mu * lap_w * S
