"""Seeded synthetic fields on the sphere mesh (workload generation).

All fields are evaluated at the mesh points in the reference's zone-0 chart
(u = latitude, v = longitude), the coordinates the reference's ``proj`` uses
(src/phelm.cpp:338-350).

* ``real_sph_harm``: orthonormal real spherical harmonics Y_l^m on the unit
  sphere (m > 0 -> cos(m lon), m < 0 -> sin(|m| lon)), by the standard
  normalised associated-Legendre recurrence.
* ``sh_field``: sum of c_lm Y_lm; ``sh_laplacian`` multiplies each degree by
  -l(l+1) (the exact spherical Laplacian).
* ``rossby_haurwitz4``: vorticity cos^4(lat) sin(lat) cos(4 lon), an l = 5
  eigenfunction of the Laplacian (stream function = -vorticity / 30).

"Amplitude" of a noise field means the coefficient vector is scaled to
Euclidean norm ``amp`` (so the field's L2 norm over the sphere is ``amp``).
"""
from __future__ import annotations

import math

import numpy as np


def _legendre_normalised(lmax: int, x: np.ndarray) -> dict:
    """Fully normalised P_l^m(x) (so that Y_lm is orthonormal), 0 <= m <= l <= lmax."""
    x = np.asarray(x, dtype=np.float64)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    P = {}
    p_mm = np.full_like(x, 1.0 / math.sqrt(4.0 * math.pi))
    for m in range(0, lmax + 1):
        if m > 0:
            p_mm = -math.sqrt((2.0 * m + 1.0) / (2.0 * m)) * s * p_mm
        P[(m, m)] = p_mm
        if m < lmax:
            p_m1 = math.sqrt(2.0 * m + 3.0) * x * p_mm
            P[(m + 1, m)] = p_m1
            a_prev, a_cur = p_mm, p_m1
            for l in range(m + 2, lmax + 1):
                a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
                b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
                nxt = a * (x * a_cur - b * a_prev)
                P[(l, m)] = nxt
                a_prev, a_cur = a_cur, nxt
    return P


def real_sph_harm(lmax: int, lat: np.ndarray, lon: np.ndarray) -> dict:
    """{(l, m): Y_lm values} for 0 <= l <= lmax, -l <= m <= l."""
    P = _legendre_normalised(lmax, np.sin(lat))
    Y = {}
    for l in range(lmax + 1):
        Y[(l, 0)] = P[(l, 0)]
        for m in range(1, l + 1):
            Y[(l, m)] = math.sqrt(2.0) * P[(l, m)] * np.cos(m * lon)
            Y[(l, -m)] = math.sqrt(2.0) * P[(l, m)] * np.sin(m * lon)
    return Y


def random_coeffs(rng: np.random.Generator, lmin: int, lmax: int, amp: float | None = None) -> dict:
    c = {}
    for l in range(lmin, lmax + 1):
        for m in range(-l, l + 1):
            c[(l, m)] = rng.standard_normal()
    if amp is not None:
        nrm = math.sqrt(sum(v * v for v in c.values()))
        c = {k: v * amp / nrm for k, v in c.items()}
    return c


def sh_field(coeffs: dict, lat, lon) -> np.ndarray:
    lmax = max(l for l, _ in coeffs)
    Y = real_sph_harm(lmax, lat, lon)
    out = np.zeros_like(np.asarray(lat, dtype=np.float64))
    for k, c in coeffs.items():
        out += c * Y[k]
    return out


def sh_laplacian(coeffs: dict) -> dict:
    return {(l, m): -l * (l + 1) * c for (l, m), c in coeffs.items()}


def sh_inverse_laplacian(coeffs: dict) -> dict:
    return {(l, m): (-c / (l * (l + 1)) if l > 0 else 0.0) for (l, m), c in coeffs.items()}


def rossby_haurwitz4(lat, lon, amp: float = 0.1) -> np.ndarray:
    """Vorticity of the wavenumber-4 Rossby-Haurwitz wave (an l = 5 mode)."""
    return amp * np.cos(lat) ** 4 * np.sin(lat) * np.cos(4.0 * lon)


def barvortex_initial(lat, lon, seed: int, lmax_noise: int = 20, amp_rh: float = 0.1,
                      amp_noise: float = 1e-3):
    """Stream function psi0 = Laplacian^{-1}(RH4 + seeded noise); returns (psi0, omega0)."""
    rng = np.random.default_rng(seed)
    c = random_coeffs(rng, 1, lmax_noise, amp_noise)
    omega = rossby_haurwitz4(lat, lon, amp_rh) + sh_field(c, lat, lon)
    psi = rossby_haurwitz4(lat, lon, amp_rh) / -30.0 + sh_field(sh_inverse_laplacian(c), lat, lon)
    return psi, omega


def laplace_problem(lat, lon, seed: int, lmax: int = 6):
    """u* = sum c_lm Y_lm (l = 1..lmax, c ~ N(0,1)); returns (u*, f = Laplacian u*)."""
    rng = np.random.default_rng(seed)
    c = random_coeffs(rng, 1, lmax)
    return sh_field(c, lat, lon), sh_field(sh_laplacian(c), lat, lon)


def coriolis_sin(lat, lon) -> np.ndarray:
    """l + h with 2 Omega = 1 and no orography: sin(latitude)."""
    return np.sin(lat)
